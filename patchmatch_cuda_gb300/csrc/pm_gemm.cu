// pm_gemm.cu -- BF16 GEMM on the fifth-generation tensor cores (tcgen05, sm_103a) for the
// learned depth proposal's convolutions (forward, data gradient and weight gradient).
//
//   C[M, N] (+)= A[M, K] . B[N, K]^T      A, B: BF16, K-major (row-major with K contiguous)
//
// One CTA of 128 threads computes a 128 x BN tile (BN <= 128, a multiple of 16) over a range
// of K tiles of 64: thread 0 streams A and B tiles into a 4-stage shared-memory ring with TMA
// (128-byte swizzle), thread 32 issues tcgen05.mma (M = 128, N = BN, K = 16 per instruction)
// into an FP32 accumulator in tensor memory and releases each stage with tcgen05.commit, and
// all four warps read the accumulator back with tcgen05.ld (warp w owns rows 32w .. 32w + 31)
// for the epilogue: BF16 store with optional bias and ReLU, FP32 store, or FP32 atomic add
// (split-K over the grid's z dimension). Every mbarrier wait is bounded: on a timeout the
// CTA records it in the error word, waits (bounded) for its own copies, frees its tensor
// memory and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "pm_internal.h"

namespace pm {
namespace {

constexpr int BM = 128, BK = 64, STAGES = 4, THREADS = 128;
constexpr int A_BYTES = BM * BK * 2;                 // 16 KB per stage
constexpr uint32_t WAIT_LIMIT = 1u << 20;           // try_wait rounds (<= 2 us each) before giving up

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, 2000;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait on phase `parity` of a barrier: false after WAIT_LIMIT unsuccessful rounds or
// once another CTA has reported a timeout in *err.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, const unsigned *err)
{
    for (uint32_t i = 0; i < WAIT_LIMIT; ++i) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((i & 63) == 63 && *(volatile const unsigned *)err) return false;
    }
    return false;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int c0, int c1,
                                            uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(bar)
        : "memory");
}

// Shared-memory matrix descriptor of a K-major tile written by TMA with the 128-byte swizzle:
// rows of 128 bytes, groups of 8 rows 1024 bytes apart (stride byte offset), version 1,
// layout SWIZZLE_128B. The leading byte offset is unused by swizzled K-major layouts.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr)
{
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
        "%11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

struct GemmArgs {
    int M, N, K;
    int bn;                 // N tile
    int k_tiles;            // K / 64
    int k_tiles_per_split;
    void *C;
    int ldc;                // elements
    int mode;               // GemmMode
    const float *bias;      // per output column, or null
    int relu;
    unsigned *err;          // set to 1 when a wait times out
};

__global__ void __launch_bounds__(THREADS, 1)
gemm_bf16_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
                 const GemmArgs g)
{
    extern __shared__ uint8_t smem_raw[];
    // 1024-byte alignment for the swizzled tiles
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int b_bytes = g.bn * BK * 2;
    const int stage_bytes = A_BYTES + b_bytes;
    uint64_t *bars = (uint64_t *)(smem + STAGES * stage_bytes);  // full[S], empty[S], done
    uint32_t *tmem_slot = (uint32_t *)(bars + 2 * STAGES + 1);
    __shared__ int s_fail;

    // a timeout elsewhere in this grid (or an earlier, unread one) ends the work at once
    if (*(volatile const unsigned *)g.err) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * g.bn;
    const int kt0 = blockIdx.z * g.k_tiles_per_split;
    const int kt1 = min(g.k_tiles, kt0 + g.k_tiles_per_split);
    const int nk = kt1 - kt0;
    int ncols = 32;
    while (ncols < g.bn) ncols <<= 1;

    if (threadIdx.x == 0) {
        s_fail = 0;
        for (int i = 0; i < STAGES; ++i) {
            mbar_init(smem_addr(bars + i), 1);
            mbar_init(smem_addr(bars + STAGES + i), 1);
        }
        mbar_init(smem_addr(bars + 2 * STAGES), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                     "r"(ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    int issued = 0;  // TMA stage loads issued by thread 0
    if (threadIdx.x == 0 && nk > 0) {
        // producer: stage s holds K tiles s, s + STAGES, ...
        for (int i = 0; i < nk; ++i) {
            const int s = i % STAGES;
            if (i >= STAGES && !mbar_wait(smem_addr(bars + STAGES + s), ((i / STAGES) - 1) & 1, g.err)) {
                atomicExch(&s_fail, 1);
                break;
            }
            if (atomicAdd(&s_fail, 0)) break;
            const uint32_t full = smem_addr(bars + s);
            uint8_t *st = smem + s * stage_bytes;
            mbar_expect_tx(full, (uint32_t)stage_bytes);
            tma_load_2d(smem_addr(st), &map_a, (kt0 + i) * BK, m0, full);
            tma_load_2d(smem_addr(st + A_BYTES), &map_b, (kt0 + i) * BK, n0, full);
            ++issued;
        }
    } else if (threadIdx.x == 32 && nk > 0) {
        // MMA issuer
        const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(g.bn >> 3) << 17) |
                               ((uint32_t)(BM >> 4) << 24);
        for (int i = 0; i < nk; ++i) {
            const int s = i % STAGES;
            if (!mbar_wait(smem_addr(bars + s), (i / STAGES) & 1, g.err)) {
                atomicExch(&s_fail, 1);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a = smem_addr(smem + s * stage_bytes);
            const uint32_t b = a + A_BYTES;
#pragma unroll
            for (int k = 0; k < BK / 16; ++k)
                mma_bf16(tmem, sw128_desc(a + 32 * k), sw128_desc(b + 32 * k), idesc,
                         (i > 0 || k > 0) ? 1u : 0u);
            mma_commit(smem_addr(bars + STAGES + s));  // frees the stage when these MMAs finish
        }
        mma_commit(smem_addr(bars + 2 * STAGES));      // accumulator complete
    }
    __syncwarp();

    // epilogue: every warp waits for the accumulator, then reads its 32 rows
    bool ok = nk > 0 && mbar_wait(smem_addr(bars + 2 * STAGES), 0, g.err);
    if (!ok && nk > 0) atomicExch(&s_fail, 1);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncthreads();
    const bool fail = s_fail != 0;
    if (!fail && nk > 0) {
        const int row = m0 + 32 * warp + lane;
        for (int c0 = 0; c0 < g.bn; c0 += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, v);
            const int col = n0 + c0;
            if (row >= g.M || col >= g.N) continue;
            if (g.bias) {
#pragma unroll
                for (int i = 0; i < 16; ++i) v[i] += g.bias[col + i];
            }
            if (g.relu) {
#pragma unroll
                for (int i = 0; i < 16; ++i) v[i] = fmaxf(v[i], 0.0f);
            }
            if (g.mode == GEMM_STORE_BF16) {
                __nv_bfloat16 *c = (__nv_bfloat16 *)g.C + (size_t)row * g.ldc + col;
                uint4 w[2];
                uint32_t *wp = (uint32_t *)w;
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
                    wp[i] = *(const uint32_t *)&h;
                }
                ((uint4 *)c)[0] = w[0];
                ((uint4 *)c)[1] = w[1];
            } else if (g.mode == GEMM_STORE_F32) {
                float *c = (float *)g.C + (size_t)row * g.ldc + col;
#pragma unroll
                for (int i = 0; i < 4; ++i) ((float4 *)c)[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
            } else {
                float *c = (float *)g.C + (size_t)row * g.ldc + col;
#pragma unroll
                for (int i = 0; i < 16; ++i) atomicAdd(c + i, v[i]);
            }
        }
    }
    if (fail && threadIdx.x == 0) {
        atomicExch(g.err, 1u);
        // let this CTA's copies land before its shared memory goes away
        for (int i = 0; i < issued && i < STAGES; ++i) {
            const int j = issued - 1 - i;
            for (uint32_t t = 0; t < WAIT_LIMIT && !mbar_try_wait(smem_addr(bars + (j % STAGES)), (j / STAGES) & 1); ++t) {
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
    }
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;

bool encode_kmajor(CUtensorMap *map, const void *base, int rows, int k, int ld, int box_rows)
{
    std::call_once(g_encode_once, [] {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    });
    if (!g_encode) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)k, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    const cuuint32_t box[2] = {BK, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return g_encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box,
                    estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

size_t gemm_smem_bytes(int bn)
{
    return (size_t)STAGES * (A_BYTES + bn * BK * 2) + 1024 + (2 * STAGES + 1) * 8 + 16;
}

// One-time host set-up (driver entry point, shared-memory opt-in): done before any stream
// capture by the callers that may capture a GEMM.
cudaError_t gemm_prepare()
{
    CUtensorMap m;
    encode_kmajor(&m, (const void *)16, 128, 64, 64, 128);  // resolves cuTensorMapEncodeTiled
    static std::once_flag attr_once;
    cudaError_t e = cudaSuccess;
    std::call_once(attr_once, [&] {
        e = cudaFuncSetAttribute(gemm_bf16_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)gemm_smem_bytes(128));
    });
    return e;
}



cudaError_t launch_gemm_bf16(const void *A, int lda, const void *B, int ldb, int M, int N, int K,
                             void *C, int ldc, int mode, const float *bias, int relu, int splits,
                             unsigned *err, cudaStream_t s)
{
    if (M <= 0 || N <= 0 || K <= 0 || M % BM || N % 16 || K % BK || lda % 8 || ldb % 8 || ldc % 8 ||
        ((uintptr_t)A & 15) || ((uintptr_t)B & 15) || ((uintptr_t)C & 15) || splits < 1)
        return cudaErrorInvalidValue;
    if (mode != GEMM_ATOMIC_F32 && splits != 1) return cudaErrorInvalidValue;
    const int bn = N < 128 ? N : 128;
    CUtensorMap ma, mb;
    if (!encode_kmajor(&ma, A, M, K, lda, BM) || !encode_kmajor(&mb, B, N, K, ldb, bn))
        return cudaErrorInvalidValue;
    GemmArgs g;
    g.M = M;
    g.N = N;
    g.K = K;
    g.bn = bn;
    g.k_tiles = K / BK;
    g.k_tiles_per_split = (g.k_tiles + splits - 1) / splits;
    g.C = C;
    g.ldc = ldc;
    g.mode = mode;
    g.bias = bias;
    g.relu = relu;
    g.err = err;
    const size_t smem = gemm_smem_bytes(bn);
    const cudaError_t pe = gemm_prepare();
    if (pe != cudaSuccess) return pe;
    const dim3 grid(M / BM, (N + bn - 1) / bn, (g.k_tiles + g.k_tiles_per_split - 1) / g.k_tiles_per_split);
    gemm_bf16_kernel<<<grid, THREADS, smem, s>>>(ma, mb, g);
    return cudaGetLastError();
}

}  // namespace pm
