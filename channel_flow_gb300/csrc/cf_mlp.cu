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
#include <vector>
#include <cmath>

#include "../../include/channel_flow_gb300.h"

namespace cf_mlp {

constexpr int BM = 128, BK = 64;
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

// STAGES: depth of the TMA ring.  Short reductions (the network's layers,
// K <= 512) use two stages, so that three CTAs fit an SM and one CTA's
// epilogue overlaps the others' loads; the long weight-gradient
// reductions (K = rows) use four.
template <int BN, int STAGES>
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
    // split K (EPI_F32 only): CTA z forms the partial product over K-slabs
    // kt0 .. kt1-1 into its own slice of the output
    const int KT = K / BK, kt0 = (int)(((long long)KT * blockIdx.z) / gridDim.z),
              kt1 = (int)(((long long)KT * (blockIdx.z + 1)) / gridDim.z);
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
        for (int kt = kt0; kt < kt1; kt++) {
            const int t = kt - kt0, s = t % STAGES;
            const uint32_t ph = (uint32_t)(t / STAGES) & 1u;
            if (t >= STAGES && !mbar_wait(saddr(&empty[s]), ph ^ 1u)) {
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
        for (int kt = kt0; kt < kt1; kt++) {
            const int t = kt - kt0, s = t % STAGES;
            const uint32_t ph = (uint32_t)(t / STAGES) & 1u;
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
                const uint32_t acc = (t | kk) != 0;
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
                    float4 *o = reinterpret_cast<float4 *>(e.outf + (size_t)blockIdx.z * M * e.ldo +
                                                           (size_t)row * e.ldo + col);
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

template <int BN, int STAGES>
static cudaError_t launch_gemm_st(const CUtensorMap &ta, const CUtensorMap &tb, int M, int N, int K,
                                  const gemm_epi &e, int *err, cudaStream_t s, int splits)
{
    constexpr size_t smem = (size_t)STAGES * (BM * BK * 2 + BN * BK * 2) + 1024;
    cudaError_t r = cudaFuncSetAttribute(k_gemm_tn<BN, STAGES>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (r != cudaSuccess) return r;
    dim3 g((unsigned)(M / BM), (unsigned)(N / BN), (unsigned)splits);
    k_gemm_tn<BN, STAGES><<<g, 128, smem, s>>>(ta, tb, M, N, K, e, err);
    return cudaGetLastError();
}

template <int BN>
static cudaError_t launch_gemm(const CUtensorMap &ta, const CUtensorMap &tb, int M, int N, int K, const gemm_epi &e,
                               int *err, cudaStream_t s, int splits = 1)
{
    return K / splits <= 512 ? launch_gemm_st<BN, 2>(ta, tb, M, N, K, e, err, s, splits)
                             : launch_gemm_st<BN, 4>(ta, tb, M, N, K, e, err, s, splits);
}

// out[i] = the sum of the split-K partials of element i, in split order
__global__ void k_splitk_sum(const float *partial, int splits, size_t n, float *out)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float v = 0.f;
    for (int z = 0; z < splits; z++) v += partial[(size_t)z * n + i];
    out[i] = v;
}

// ---------------------------------------------------------------------------
// MLP data movement and training kernels (FP32 / BF16, device pointers)

constexpr int MLP_IN = 270, MLP_K1 = 320, MLP_H = 128, MLP_OUT = 5, MLP_N3 = 16, MLP_K3 = 64;

struct mlp_grid {
    int X, Y, Z;            // interior cells
    __host__ __device__ int Ym() const { return Y + 4; }
    __host__ __device__ int Zm() const { return Z + 4; }
    // interior cell r (x-major, z fastest) -> field index
    __host__ __device__ size_t cell(long long r) const
    {
        const int k = (int)(r % Z), j = (int)((r / Z) % Y), i = (int)(r / ((long long)Z * Y));
        return ((size_t)(i + 3) * Ym() + (j + 2)) * Zm() + (k + 2);
    }
};

struct mlp_levels {
    const double *u[3][5];  // U^n, U^{n-1}, U^{n-2}
};

// features of row r: for kind l (0: the first time difference
// U^n - U^(n-1), over scale[v]; 1: the second difference U^n - 2 U^(n-1) +
// U^(n-2), over scale[5 + v]), variable v and neighbour s of the 3x3x3
// stencil (s = 9 (di+1) + 3 (dj+1) + (dk+1)), column 135 l + 27 v + s;
// columns 270..319 are zero.  The second difference is formed in FP64
// before the BF16 rounding, so the features resolve it at BF16 precision
// relative to its own size.  One thread writes 8 columns (16 bytes).
__global__ void k_mlp_features(mlp_grid g, mlp_levels L, const float *scale, const int *rows, long long M,
                               long long Mpad, __nv_bfloat16 *X)
{
    constexpr int CH = MLP_K1 / 8;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long r = t / CH;
    const int ch = (int)(t % CH);
    if (r >= Mpad) return;
    __align__(16) __nv_bfloat16 h[8];
    if (r >= M || ch * 8 >= MLP_IN) {
#pragma unroll
        for (int e = 0; e < 8; e++) h[e] = __float2bfloat16(0.f);
    } else {
        const size_t q = g.cell(rows ? rows[r] : r);
        const ptrdiff_t sx = (ptrdiff_t)g.Ym() * g.Zm(), sy = g.Zm();
#pragma unroll
        for (int e = 0; e < 8; e++) {
            const int c = ch * 8 + e;
            float f = 0.f;
            if (c < MLP_IN) {
                const int l = c / 135, rem = c % 135, v = rem / 27, st = rem % 27;
                const ptrdiff_t p = (ptrdiff_t)q + (st / 9 - 1) * sx + ((st / 3) % 3 - 1) * sy + (st % 3 - 1);
                const double a0 = L.u[0][v][p], a1 = L.u[1][v][p];
                const double d = l == 0 ? a0 - a1 : (a0 - 2.0 * a1) + L.u[2][v][p];
                f = (float)d * (1.0f / scale[5 * l + v]);
            }
            h[e] = __float2bfloat16(f);
        }
    }
    *reinterpret_cast<uint4 *>(X + (size_t)r * MLP_K1 + ch * 8) = *reinterpret_cast<const uint4 *>(h);
}

// Feature rows of every interior cell in two passes (the guess on the
// whole grid).  k_mlp_diffs forms the ten time differences of every array
// index once, rounded to FP32 as k_mlp_features rounds them: D[y * N + q],
// y < 5 the first difference of variable y, y >= 5 the second difference
// of variable y - 5.  k_mlp_features_grid then gathers the 270 stencil
// values of 32 consecutive rows per block into shared memory (one lane per
// row, so each gather is coalesced along z) and writes the block's 32 rows
// (20 KB, contiguous in X) with coalesced stores.  The values equal
// k_mlp_features' bit for bit: the same FP64 differences, the same FP32
// rounding and scaling.
__global__ void __launch_bounds__(256) k_mlp_diffs(size_t N, mlp_levels L, float *D)
{
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= N) return;
#pragma unroll
    for (int v = 0; v < 5; v++) {
        const double a0 = L.u[0][v][q], a1 = L.u[1][v][q], a2 = L.u[2][v][q];
        D[(size_t)v * N + q] = (float)(a0 - a1);
        D[(size_t)(5 + v) * N + q] = (float)((a0 - 2.0 * a1) + a2);
    }
}

constexpr int MLP_FROWS = 32;                 // rows per block
constexpr int MLP_FPAIRS = MLP_K1 / 2;        // 160 32-bit words per row
constexpr int MLP_FSTRIDE = MLP_K1 + 2;       // padded row stride in bf16: 161 words, lanes hit distinct banks
constexpr int MLP_FWARPS = 10;                // one warp per (kind, variable)

// Ten warps per block, warp w gathering the 27 stencil columns of kind
// l = w / 5, variable v = w % 5 for the block's 32 rows (one lane per row),
// the stencil offsets unrolled as constants; each warp also clears five of
// the fifty padding columns.
__global__ void __launch_bounds__(32 * MLP_FWARPS) k_mlp_features_grid(mlp_grid g, size_t N, const float *__restrict__ D,
                                                                      const float *scale, long long M, long long Mpad,
                                                                      uint32_t *Xw)
{
    __shared__ __align__(16) __nv_bfloat16 tile[MLP_FROWS * MLP_FSTRIDE];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long r0 = (long long)blockIdx.x * MLP_FROWS;
    const long long r = r0 + lane;
    const bool live = r < M;
    const int l = warp / 5, v = warp % 5;
    const float inv = 1.0f / scale[5 * l + v];
    __nv_bfloat16 *row = tile + lane * MLP_FSTRIDE + 135 * l + 27 * v;
    if (live) {
        const ptrdiff_t sx = (ptrdiff_t)g.Ym() * g.Zm(), sy = g.Zm();
        const float *src = D + (size_t)(5 * l + v) * N + g.cell(r);
#pragma unroll
        for (int st = 0; st < 27; st++) {
            const ptrdiff_t off = (st / 9 - 1) * sx + ((st / 3) % 3 - 1) * sy + (st % 3 - 1);
            row[st] = __float2bfloat16(src[off] * inv);
        }
    } else {
#pragma unroll
        for (int st = 0; st < 27; st++) row[st] = __float2bfloat16(0.f);
    }
#pragma unroll
    for (int e = 0; e < 5; e++) tile[lane * MLP_FSTRIDE + MLP_IN + 5 * warp + e] = __float2bfloat16(0.f);
    __syncthreads();
    const long long rows = Mpad - r0 < MLP_FROWS ? Mpad - r0 : MLP_FROWS;
    const uint32_t *t32 = reinterpret_cast<const uint32_t *>(tile);
    for (int w = threadIdx.x; w < rows * MLP_FPAIRS; w += blockDim.x) {
        const int rr = w / MLP_FPAIRS, pr = w % MLP_FPAIRS;
        Xw[(size_t)r0 * MLP_FPAIRS + w] = t32[rr * (MLP_FSTRIDE / 2) + pr];
    }
}

// coefficients of the linear predictor P = U^n + a_v dU^n + b_v d2U of
// U^(n+1) that the network corrects (a = b = 1: the quadratic extrapolation)
struct mlp_coef {
    double a[5], b[5];
};

// targets of row r: the error U^(n+1) - P of the predictor, over
// scale[5 + v] * oscale[v]; columns 5..15 zero.  L.u[0..2] = U^n, U^(n-1),
// U^(n-2), next = U^(n+1)
__global__ void k_mlp_targets(mlp_grid g, mlp_levels L, mlp_levels next, mlp_coef cf, const float *scale,
                              const float *oscale, const int *rows, long long M, long long Mpad, float *T)
{
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= Mpad) return;
    float *t = T + (size_t)r * MLP_N3;
    for (int c = 0; c < MLP_N3; c++) t[c] = 0.f;
    if (r >= M) return;
    const size_t q = g.cell(rows ? rows[r] : r);
    for (int v = 0; v < 5; v++) {
        const double un = L.u[0][v][q], u1 = L.u[1][v][q];
        const double d1 = un - u1, d2 = (un - 2.0 * u1) + L.u[2][v][q];
        const double e = ((next.u[0][v][q] - un) - cf.a[v] * d1) - cf.b[v] * d2;
        t[v] = (float)(e / ((double)scale[5 + v] * (double)oscale[v]));
    }
}

// the learned initial guess on every interior cell:
// U_ = P + scale[5 + v] * oscale[v] * Y (Y null: the predictor alone)
__global__ void k_mlp_apply(mlp_grid g, mlp_levels L, mlp_coef cf, const float *scale, const float *oscale,
                            const float *Y, long long M, double *o0, double *o1, double *o2, double *o3, double *o4)
{
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= M) return;
    const size_t q = g.cell(r);
    double *o[5] = {o0, o1, o2, o3, o4};
#pragma unroll
    for (int v = 0; v < 5; v++) {
        const double un = L.u[0][v][q], u1 = L.u[1][v][q];
        const double d1 = un - u1, d2 = (un - 2.0 * u1) + L.u[2][v][q];
        const double c = Y ? (double)scale[5 + v] * (double)oscale[v] * (double)Y[(size_t)r * MLP_N3 + v] : 0.0;
        o[v][q] = ((un + cf.a[v] * d1) + cf.b[v] * d2) + c;
    }
}

// partial sums (block b of row y of the grid) of squared time differences
// over the interior: D = 1: y < 5 the first difference U^n - U^(n-1) of
// variable y, y >= 5 the second difference U^n - 2 U^(n-1) + U^(n-2) of
// variable y - 5 (levels L.u[0..2]); D = 3: the third difference
// U^(n+1) - 3 U^n + 3 U^(n-1) - U^(n-2) of variable y (levels L.u[0..3])
struct mlp_levels4 {
    const double *u[4][5];
};

template <int D>
__global__ void k_mlp_sq_partial(mlp_grid g, mlp_levels4 L, long long M, double *partial)
{
    const int y = blockIdx.y, v = D == 1 ? y % 5 : y;
    const bool second = D == 1 && y >= 5;
    double s = 0;
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < M; r += (long long)gridDim.x * blockDim.x) {
        const size_t q = g.cell(r);
        double d;
        if (D == 3) d = L.u[0][v][q] - 3.0 * L.u[1][v][q] + 3.0 * L.u[2][v][q] - L.u[3][v][q];
        else if (second) d = (L.u[0][v][q] - 2.0 * L.u[1][v][q]) + L.u[2][v][q];
        else d = L.u[0][v][q] - L.u[1][v][q];
        s += d * d;
    }
    __shared__ double sh[256];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[(size_t)y * gridDim.x + blockIdx.x] = sh[0];
}

// partial sums (block b, variable v) of the least-squares fit of the
// predictor: d1 d1, d1 d2, d2 d2, t d1, t d2, t t with d1 = U^n - U^(n-1),
// d2 = U^n - 2 U^(n-1) + U^(n-2), t = U^(n+1) - U^n (L.u[0..3] = U^(n+1),
// U^n, U^(n-1), U^(n-2)); partial[(b * 5 + v) * 6 + s]
struct mlp_levels20 {
    const double *u[4][5];
};

__global__ void k_mlp_base_sums(mlp_grid g, mlp_levels20 L, long long M, double *partial)
{
    const int v = blockIdx.y;
    double s[6] = {0, 0, 0, 0, 0, 0};
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < M; r += (long long)gridDim.x * blockDim.x) {
        const size_t q = g.cell(r);
        const double un = L.u[1][v][q], u1 = L.u[2][v][q];
        const double d1 = un - u1, d2 = (un - 2.0 * u1) + L.u[3][v][q], t = L.u[0][v][q] - un;
        s[0] += d1 * d1;
        s[1] += d1 * d2;
        s[2] += d2 * d2;
        s[3] += t * d1;
        s[4] += t * d2;
        s[5] += t * t;
    }
    __shared__ double sh[6][256];
#pragma unroll
    for (int c = 0; c < 6; c++) sh[c][threadIdx.x] = s[c];
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
#pragma unroll
            for (int c = 0; c < 6; c++) sh[c][threadIdx.x] += sh[c][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < 6) partial[((size_t)blockIdx.x * 5 + v) * 6 + threadIdx.x] = sh[threadIdx.x][0];
}

// the feature scales on the device (no host round trip): scale[y] =
// sqrt(sum over the nb partial sums of row y / M), 1 where that is 0; one
// warp per row, lane-strided sums and a shuffle tree
__global__ void k_mlp_scale_finish(const double *partial, int nb, long long M, float *scale)
{
    const int y = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (y >= 10) return;
    double t = 0;
    for (int b = lane; b < nb; b += 32) t += partial[(size_t)y * nb + b];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) {
        const double r = sqrt(t / (double)M);
        scale[y] = r > 0 ? (float)r : 1.0f;
    }
}

// per-block sums over rows of T.Y, Y.Y and T.T for each of the 5 outputs
// (FP64): partial[(b * 3 + s) * 5 + v]
__global__ void k_mlp_dot_partial(const float *Y, const float *T, long long M, double *partial)
{
    double ty[5] = {0, 0, 0, 0, 0}, yy[5] = {0, 0, 0, 0, 0}, tt[5] = {0, 0, 0, 0, 0};
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < M; r += (long long)gridDim.x * blockDim.x)
#pragma unroll
        for (int v = 0; v < 5; v++) {
            const double y = Y[(size_t)r * MLP_N3 + v], t = T[(size_t)r * MLP_N3 + v];
            ty[v] += t * y;
            yy[v] += y * y;
            tt[v] += t * t;
        }
    __shared__ double sh[15][256];
    for (int v = 0; v < 5; v++) {
        sh[v][threadIdx.x] = ty[v];
        sh[5 + v][threadIdx.x] = yy[v];
        sh[10 + v][threadIdx.x] = tt[v];
    }
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int n = 0; n < 15; n++) sh[n][threadIdx.x] += sh[n][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < 15) partial[(size_t)blockIdx.x * 15 + threadIdx.x] = sh[threadIdx.x][0];
}

// dL/dY of the mean squared error over the 5 outputs of M rows: dY (bf16,
// [Mpad x 64], columns >= 5 zero), its transpose dYT ([16 x Mpad]), and
// per-block loss and db3 partial sums
__global__ void k_mlp_loss_grad(const float *Y, const float *T, long long M, long long Mpad, __nv_bfloat16 *dY,
                                __nv_bfloat16 *dYT, float *partial)
{
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0, db[5] = {0, 0, 0, 0, 0};
    if (r < Mpad) {
        const float sc = 2.0f / (float)(M * MLP_OUT);
        for (int c = 0; c < MLP_K3; c++) {
            float gv = 0.f;
            if (c < MLP_OUT && r < M) {
                const float d = Y[(size_t)r * MLP_N3 + c] - T[(size_t)r * MLP_N3 + c];
                l += d * d;
                gv = sc * d;
                db[c] = gv;
            }
            dY[(size_t)r * MLP_K3 + c] = __float2bfloat16(gv);
            if (c < MLP_N3) dYT[(size_t)c * Mpad + r] = __float2bfloat16(gv);
        }
    }
    __shared__ float sh[6][256];
    sh[0][threadIdx.x] = l;
    for (int c = 0; c < 5; c++) sh[1 + c][threadIdx.x] = db[c];
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int n = 0; n < 6; n++) sh[n][threadIdx.x] += sh[n][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int n = 0; n < 6; n++) partial[(size_t)blockIdx.x * 6 + n] = sh[n][0];
}

// dZ = dH * SiLU'(Z), both as rows [Mpad x 128] and transposed [128 x Mpad]
// (32 x 32 tiles through shared memory); partial column sums for the bias
__global__ void k_mlp_silu_bwd(const float *dH, const float *Z, long long Mpad, __nv_bfloat16 *dZ,
                               __nv_bfloat16 *dZT)
{
    __shared__ __nv_bfloat16 tile[32][33];
    const long long r0 = (long long)blockIdx.x * 32;
    const int c0 = blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;      // 32 x 8
    for (int yy = ty; yy < 32; yy += 8) {
        const long long r = r0 + yy;
        const int c = c0 + tx;
        const size_t i = (size_t)r * MLP_H + c;
        const float z = Z[i];
        const float sgm = 1.0f / (1.0f + __expf(-z));
        const float gz = dH[i] * (sgm * (1.0f + z * (1.0f - sgm)));
        const __nv_bfloat16 h = __float2bfloat16(gz);
        dZ[i] = h;
        tile[yy][tx] = h;
    }
    __syncthreads();
    for (int yy = ty; yy < 32; yy += 8) dZT[(size_t)(c0 + yy) * Mpad + r0 + tx] = tile[tx][yy];
}

// dst [cols x rows] = src [rows x cols]^T (bf16, rows multiple of 32, cols multiple of 32)
__global__ void k_transpose_bf16(const __nv_bfloat16 *src, long long rows, int cols, __nv_bfloat16 *dst)
{
    __shared__ __nv_bfloat16 tile[32][33];
    const long long r0 = (long long)blockIdx.x * 32;
    const int c0 = blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (int yy = ty; yy < 32; yy += 8) tile[yy][tx] = src[(size_t)(r0 + yy) * cols + c0 + tx];
    __syncthreads();
    for (int yy = ty; yy < 32; yy += 8) dst[(size_t)(c0 + yy) * rows + r0 + tx] = tile[tx][yy];
}

// column sums of a bf16 [rows x cols] matrix into out[cols] (fp32); one block per column
__global__ void k_colsum_bf16(const __nv_bfloat16 *src, long long rows, int cols, float *out)
{
    const int c = blockIdx.x;
    float s = 0;
    for (long long r = threadIdx.x; r < rows; r += blockDim.x) s += __bfloat162float(src[(size_t)r * cols + c]);
    __shared__ float sh[256];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[c] = sh[0];
}

// Adam step on n parameters (bias-corrected)
__global__ void k_adam(float *p, const float *gr, float *m, float *v, long long n, float lr, float b1, float b2,
                       float eps, float c1, float c2)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const float g = gr[t];
    const float mm = b1 * m[t] + (1 - b1) * g;
    const float vv = b2 * v[t] + (1 - b2) * g * g;
    m[t] = mm;
    v[t] = vv;
    p[t] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
}

// fp32 parameters -> the BF16 operand layouts of the forward and backward GEMMs:
// W1b [128 x 320], W2b [128 x 128], W3b [16 x 128] = W3T^T, W2T [128 x 128] = W2^T,
// W3p [128 x 64] with W3p[h][o] = W3T[h][o] (o < 16), zero beyond
__global__ void k_mlp_pack(const float *W1, const float *W2, const float *W3T, __nv_bfloat16 *W1b,
                           __nv_bfloat16 *W2b, __nv_bfloat16 *W3b, __nv_bfloat16 *W2T, __nv_bfloat16 *W3p)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < MLP_H * MLP_K1) W1b[t] = __float2bfloat16(W1[t]);
    if (t < MLP_H * MLP_H) {
        const int a = t / MLP_H, b = t % MLP_H;
        W2b[t] = __float2bfloat16(W2[t]);
        W2T[(size_t)b * MLP_H + a] = __float2bfloat16(W2[t]);
    }
    if (t < MLP_N3 * MLP_H) {
        const int o = t / MLP_H, h = t % MLP_H;
        W3b[t] = __float2bfloat16(W3T[(size_t)h * MLP_N3 + o]);
    }
    if (t < MLP_H * MLP_K3) {
        const int h = t / MLP_K3, o = t % MLP_K3;
        W3p[t] = __float2bfloat16(o < MLP_N3 ? W3T[(size_t)h * MLP_N3 + o] : 0.f);
    }
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

// C = A B^T in FP32 with K split over `splits` CTAs per output tile
// (see channel_flow_gb300.h)
int cf_gemm_bf16_splitk(void *stream, const void *A, const void *B, int M, int N, int K, int splits,
                        float *partial, float *out, int *err_dev)
{
    if (!A || !B || !out || !partial || !err_dev || splits < 1) return CF_ERR_ARG;
    if (M <= 0 || N <= 0 || K <= 0 || M % BM || K % BK || N % 16 || splits > K / BK) return CF_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) & 15) return CF_ERR_ARG;
    int bn = 0;
    for (int c : {256, 128, 64, 32, 16})
        if (N % c == 0) { bn = c; break; }
    CUtensorMap ta, tb;
    if (!make_map(&ta, A, M, K, BM) || !make_map(&tb, B, N, K, bn)) return CF_ERR_CUDA;
    gemm_epi e{EPI_F32, nullptr, partial, nullptr, nullptr, N};
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t r;
    switch (bn) {
    case 256: r = launch_gemm<256>(ta, tb, M, N, K, e, err_dev, s, splits); break;
    case 128: r = launch_gemm<128>(ta, tb, M, N, K, e, err_dev, s, splits); break;
    case 64: r = launch_gemm<64>(ta, tb, M, N, K, e, err_dev, s, splits); break;
    case 32: r = launch_gemm<32>(ta, tb, M, N, K, e, err_dev, s, splits); break;
    default: r = launch_gemm<16>(ta, tb, M, N, K, e, err_dev, s, splits); break;
    }
    if (r != cudaSuccess) return CF_ERR_CUDA;
    const size_t n = (size_t)M * N;
    k_splitk_sum<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(partial, splits, n, out);
    return cudaGetLastError() == cudaSuccess ? CF_OK : CF_ERR_CUDA;
}

static mlp_levels levels(const double *const *u15)
{
    mlp_levels L;
    for (int l = 0; l < 3; l++)
        for (int v = 0; v < 5; v++) L.u[l][v] = u15 ? u15[5 * l + v] : nullptr;
    return L;
}

static inline unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

// features [Mpad x 320] bf16 of M interior rows (rows = NULL: all cells in order)
int cf_mlp_features(void *stream, int X, int Y, int Z, const double *const *levels15, const float *scale,
                    const int *rows, long long M, long long Mpad, void *Xout)
{
    if (!levels15 || !scale || !Xout || M <= 0 || Mpad < M || Mpad % 128) return CF_ERR_ARG;
    mlp_grid g{X, Y, Z};
    k_mlp_features<<<nblk(Mpad * (MLP_K1 / 8), 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        g, levels(levels15), scale, rows, M, Mpad, static_cast<__nv_bfloat16 *>(Xout));
    return cudaGetLastError() == cudaSuccess ? CF_OK : CF_ERR_CUDA;
}

int cf_mlp_features_grid(void *stream, int X, int Y, int Z, const double *const *levels15, const float *scale,
                         long long Mpad, float *diff_scratch, void *Xout)
{
    const long long M = (long long)X * Y * Z;
    if (!levels15 || !scale || !Xout || !diff_scratch || X <= 0 || Y <= 0 || Z <= 0 || Mpad < M || Mpad % 128)
        return CF_ERR_ARG;
    for (int i = 0; i < 15; i++)
        if (!levels15[i]) return CF_ERR_ARG;
    mlp_grid g{X, Y, Z};
    const size_t N = (size_t)(X + 6) * g.Ym() * g.Zm();
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    k_mlp_diffs<<<nblk((long long)N, 256), 256, 0, s>>>(N, levels(levels15), diff_scratch);
    k_mlp_features_grid<<<nblk(Mpad, MLP_FROWS), 32 * MLP_FWARPS, 0, s>>>(g, N, diff_scratch, scale, M, Mpad,
                                                                          static_cast<uint32_t *>(Xout));
    return cudaGetLastError() == cudaSuccess ? CF_OK : CF_ERR_CUDA;
}

// targets [Mpad x 16] fp32: levels20 = U^(n+1), U^n, U^(n-1), U^(n-2)
static mlp_coef coef_of(const double *c10)
{
    mlp_coef c;
    for (int v = 0; v < 5; v++) {
        c.a[v] = c10 ? c10[v] : 1.0;
        c.b[v] = c10 ? c10[5 + v] : 1.0;
    }
    return c;
}

int cf_mlp_targets(void *stream, int X, int Y, int Z, const double *const *levels20, const double *coef10,
                   const float *scale, const float *oscale, const int *rows, long long M, long long Mpad, float *T)
{
    if (!levels20 || !scale || !oscale || !T || M <= 0 || Mpad < M || Mpad % 128) return CF_ERR_ARG;
    mlp_grid g{X, Y, Z};
    mlp_levels next{}, L{};
    for (int v = 0; v < 5; v++) next.u[0][v] = levels20[v];
    for (int l = 0; l < 3; l++)
        for (int v = 0; v < 5; v++) L.u[l][v] = levels20[5 * (l + 1) + v];
    k_mlp_targets<<<nblk(Mpad, 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(g, L, next, coef_of(coef10), scale,
                                                                                   oscale, rows, M, Mpad, T);
    return cudaGetLastError() == cudaSuccess ? CF_OK : CF_ERR_CUDA;
}

// U_ (out5) = P + scale * oscale * Y on all interior cells; levels15 = U^n,
// U^(n-1), U^(n-2)
int cf_mlp_apply(void *stream, int X, int Y, int Z, const double *const *levels15, const double *coef10,
                 const float *scale, const float *oscale, const float *Yp, double *const *out5)
{
    if (!levels15 || !out5 || (Yp && (!scale || !oscale))) return CF_ERR_ARG;
    mlp_grid g{X, Y, Z};
    const long long M = (long long)X * Y * Z;
    k_mlp_apply<<<nblk(M, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        g, levels(levels15), coef_of(coef10), scale, oscale, Yp, M, out5[0], out5[1], out5[2], out5[3], out5[4]);
    return cudaGetLastError() == cudaSuccess ? CF_OK : CF_ERR_CUDA;
}

int cf_mlp_base_sums(void *stream, int X, int Y, int Z, const double *const *levels20, double *partial_dev,
                     int nblocks, double *sums30)
{
    if (!levels20 || !partial_dev || !sums30 || nblocks <= 0 || X <= 0 || Y <= 0 || Z <= 0) return CF_ERR_ARG;
    mlp_grid g{X, Y, Z};
    mlp_levels20 L{};
    for (int l = 0; l < 4; l++)
        for (int v = 0; v < 5; v++) {
            if (!levels20[5 * l + v]) return CF_ERR_ARG;
            L.u[l][v] = levels20[5 * l + v];
        }
    const long long M = (long long)X * Y * Z;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    k_mlp_base_sums<<<dim3((unsigned)nblocks, 5), 256, 0, s>>>(g, L, M, partial_dev);
    std::vector<double> h((size_t)30 * nblocks);
    if (cudaMemcpyAsync(h.data(), partial_dev, h.size() * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return CF_ERR_CUDA;
    for (int n = 0; n < 30; n++) {
        double t = 0;
        for (int b = 0; b < nblocks; b++) t += h[(size_t)b * 30 + n];
        sums30[n] = t;
    }
    return CF_OK;
}

static int mlp_rms(int D, void *stream, int X, int Y, int Z, const double *const *lv, double *partial_dev,
                   int nblocks, double *rms)
{
    if (!lv || !partial_dev || !rms || nblocks <= 0 || X <= 0 || Y <= 0 || Z <= 0) return CF_ERR_ARG;
    mlp_grid g{X, Y, Z};
    mlp_levels4 L{};
    const int nlev = D == 1 ? 3 : 4, nrow = D == 1 ? 10 : 5;
    for (int l = 0; l < nlev; l++)
        for (int v = 0; v < 5; v++) {
            if (!lv[5 * l + v]) return CF_ERR_ARG;
            L.u[l][v] = lv[5 * l + v];
        }
    const long long M = (long long)X * Y * Z;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (D == 1) k_mlp_sq_partial<1><<<dim3((unsigned)nblocks, nrow), 256, 0, s>>>(g, L, M, partial_dev);
    else k_mlp_sq_partial<3><<<dim3((unsigned)nblocks, nrow), 256, 0, s>>>(g, L, M, partial_dev);
    std::vector<double> h((size_t)nrow * nblocks);
    if (cudaMemcpyAsync(h.data(), partial_dev, h.size() * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return CF_ERR_CUDA;
    for (int y = 0; y < nrow; y++) {
        double t = 0;
        for (int b = 0; b < nblocks; b++) t += h[(size_t)y * nblocks + b];
        rms[y] = std::sqrt(t / (double)M);
    }
    return CF_OK;
}

// RMS over the interior per variable of the first (rms10[0..4]) and second
// (rms10[5..9]) time differences; levels15 = U^n, U^(n-1), U^(n-2)
int cf_mlp_rms(void *stream, int X, int Y, int Z, const double *const *levels15, double *partial_dev,
               int nblocks, double *rms10)
{
    return mlp_rms(1, stream, X, Y, Z, levels15, partial_dev, nblocks, rms10);
}

// the ten feature scales of cf_mlp_rms written to scale10_dev on the
// device, stream-ordered (no synchronisation)
int cf_mlp_scale(void *stream, int X, int Y, int Z, const double *const *lv, double *partial_dev, int nblocks,
                 float *scale10_dev)
{
    if (!lv || !partial_dev || !scale10_dev || nblocks <= 0 || X <= 0 || Y <= 0 || Z <= 0) return CF_ERR_ARG;
    mlp_grid g{X, Y, Z};
    mlp_levels4 L{};
    for (int l = 0; l < 3; l++)
        for (int v = 0; v < 5; v++) {
            if (!lv[5 * l + v]) return CF_ERR_ARG;
            L.u[l][v] = lv[5 * l + v];
        }
    const long long M = (long long)X * Y * Z;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    k_mlp_sq_partial<1><<<dim3((unsigned)nblocks, 10), 256, 0, s>>>(g, L, M, partial_dev);
    k_mlp_scale_finish<<<1, 320, 0, s>>>(partial_dev, nblocks, M, scale10_dev);
    return cudaGetLastError() == cudaSuccess ? CF_OK : CF_ERR_CUDA;
}

// RMS of U^(n+1) - 3 U^n + 3 U^(n-1) - U^(n-2) per variable (levels20 in that order)
int cf_mlp_rms3(void *stream, int X, int Y, int Z, const double *const *levels20, double *partial_dev,
                int nblocks, double *rms5)
{
    return mlp_rms(3, stream, X, Y, Z, levels20, partial_dev, nblocks, rms5);
}

// sums over M rows of T.Y, Y.Y and T.T per output into sums15 (host):
// [0..4] = T.Y, [5..9] = Y.Y, [10..14] = T.T
int cf_mlp_dot(void *stream, const float *Yv, const float *T, long long M, double *partial_dev, int nblocks,
               double *sums15)
{
    if (!Yv || !T || !partial_dev || !sums15 || M <= 0 || nblocks <= 0) return CF_ERR_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    k_mlp_dot_partial<<<(unsigned)nblocks, 256, 0, s>>>(Yv, T, M, partial_dev);
    std::vector<double> h((size_t)15 * nblocks);
    if (cudaMemcpyAsync(h.data(), partial_dev, h.size() * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return CF_ERR_CUDA;
    for (int n = 0; n < 15; n++) {
        double t = 0;
        for (int b = 0; b < nblocks; b++) t += h[(size_t)b * 15 + n];
        sums15[n] = t;
    }
    return CF_OK;
}

int cf_mlp_loss_grad(void *stream, const float *Yv, const float *T, long long M, long long Mpad, void *dY, void *dYT,
                     float *partial)
{
    if (!Yv || !T || !dY || !dYT || !partial || Mpad % 256) return CF_ERR_ARG;
    k_mlp_loss_grad<<<nblk(Mpad, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        Yv, T, M, Mpad, static_cast<__nv_bfloat16 *>(dY), static_cast<__nv_bfloat16 *>(dYT), partial);
    return cudaGetLastError() == cudaSuccess ? CF_OK : CF_ERR_CUDA;
}

int cf_mlp_silu_bwd(void *stream, const float *dH, const float *Zv, long long Mpad, void *dZ, void *dZT)
{
    if (!dH || !Zv || !dZ || !dZT || Mpad % 32) return CF_ERR_ARG;
    k_mlp_silu_bwd<<<dim3((unsigned)(Mpad / 32), MLP_H / 32), dim3(32, 8), 0, static_cast<cudaStream_t>(stream)>>>(
        dH, Zv, Mpad, static_cast<__nv_bfloat16 *>(dZ), static_cast<__nv_bfloat16 *>(dZT));
    return cudaGetLastError() == cudaSuccess ? CF_OK : CF_ERR_CUDA;
}

int cf_transpose_bf16(void *stream, const void *src, long long rows, int cols, void *dst)
{
    if (!src || !dst || rows % 32 || cols % 32) return CF_ERR_ARG;
    k_transpose_bf16<<<dim3((unsigned)(rows / 32), (unsigned)(cols / 32)), dim3(32, 8), 0,
                       static_cast<cudaStream_t>(stream)>>>(static_cast<const __nv_bfloat16 *>(src), rows, cols,
                                                            static_cast<__nv_bfloat16 *>(dst));
    return cudaGetLastError() == cudaSuccess ? CF_OK : CF_ERR_CUDA;
}

int cf_colsum_bf16(void *stream, const void *src, long long rows, int cols, float *out)
{
    if (!src || !out) return CF_ERR_ARG;
    k_colsum_bf16<<<(unsigned)cols, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const __nv_bfloat16 *>(src), rows, cols, out);
    return cudaGetLastError() == cudaSuccess ? CF_OK : CF_ERR_CUDA;
}

int cf_adam(void *stream, float *p, const float *g, float *m, float *v, long long n, float lr, float b1, float b2,
            float eps, int t)
{
    if (!p || !g || !m || !v || n <= 0 || t < 1) return CF_ERR_ARG;
    const float c1 = 1.f - std::pow(b1, (float)t), c2 = 1.f - std::pow(b2, (float)t);
    k_adam<<<nblk(n, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(p, g, m, v, n, lr, b1, b2, eps, c1, c2);
    return cudaGetLastError() == cudaSuccess ? CF_OK : CF_ERR_CUDA;
}

int cf_mlp_pack(void *stream, const float *W1, const float *W2, const float *W3, void *W1b, void *W2b, void *W3b,
                void *W2T, void *W3p)
{
    if (!W1 || !W2 || !W3 || !W1b || !W2b || !W3b || !W2T || !W3p) return CF_ERR_ARG;
    k_mlp_pack<<<nblk(MLP_H * MLP_K1, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        W1, W2, W3, static_cast<__nv_bfloat16 *>(W1b), static_cast<__nv_bfloat16 *>(W2b),
        static_cast<__nv_bfloat16 *>(W3b), static_cast<__nv_bfloat16 *>(W2T), static_cast<__nv_bfloat16 *>(W3p));
    return cudaGetLastError() == cudaSuccess ? CF_OK : CF_ERR_CUDA;
}

}  // extern "C"
