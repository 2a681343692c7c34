// Tensor-core (tcgen05) GEMM of the library: D = A * B^T with bf16 operands and
// FP32 accumulation in tensor memory.  It is the contraction the learned
// coarse-slice closure's convolutions are built on, and it is exported
// (msl_tc_gemm_bf16) so the descriptor and tensor-memory conventions of
// msl_tc.cuh are checked on their own against a plain FP32 reference.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "msl_internal.h"
#include "msl_tc.cuh"

namespace msl {

namespace {

constexpr int kTcM = 128;        // rows per CTA tile (one MMA's M)
constexpr int kTcK = 64;         // K per shared-memory stage (one 128-byte row)
constexpr uint32_t kTcWait = 1u << 22;

// One CTA per 128-row tile of D.  Each K stage: the 128 threads copy the A tile
// (128 x 64) and the B tile (N x 64) into 128B-swizzled shared memory, one thread
// issues four K = 16 MMAs into the TMEM accumulator and commits them to an
// mbarrier, everyone waits, then the next stage reuses the tiles.  At the end
// each warp reads its 32 TMEM lanes (its 32 rows of D) 16 columns at a time.
__global__ void __launch_bounds__(128) tc_gemm_kernel(const __nv_bfloat16 *__restrict__ A,
                                                      const __nv_bfloat16 *__restrict__ B, float *__restrict__ D,
                                                      int M, int N, int K, int ncols, int *err) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *base = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char *sa = base;                       // 16 KB
    unsigned char *sb = base + kTcM * kTcK * 2;     // N x 128 bytes
    __shared__ uint64_t bar;
    __shared__ uint32_t tmem_base;
    __shared__ int failed;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * kTcM;
    if (warp == 0) tc::tmem_alloc(&tmem_base, (uint32_t)ncols);
    if (tid == 0) {
        mbar_init(&bar, 1);
        mbar_fence_init();
        failed = 0;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_base;
    const uint32_t idesc = tc::idesc_bf16(kTcM, N);
    uint32_t phase = 0;
    for (int k0 = 0; k0 < K; k0 += kTcK) {
        // 16-byte chunks: row r, chunk c (8 bf16)
        for (int i = tid; i < kTcM * 8; i += 128) {
            const int r = i >> 3, c = i & 7;
            const uint4 v = *(const uint4 *)(A + (size_t)(m0 + r) * K + k0 + c * 8);
            *(uint4 *)(sa + tc::sw128_offset(r, c * 8)) = v;
        }
        for (int i = tid; i < N * 8; i += 128) {
            const int r = i >> 3, c = i & 7;
            const uint4 v = *(const uint4 *)(B + (size_t)r * K + k0 + c * 8);
            *(uint4 *)(sb + tc::sw128_offset(r, c * 8)) = v;
        }
        fence_proxy_async();  // the generic-proxy tile writes, visible to the tensor core
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
#pragma unroll
            for (int kk = 0; kk < kTcK / 16; ++kk) {
                const uint64_t da = tc::desc_sw128(smem_u32(sa) + kk * 32);
                const uint64_t db = tc::desc_sw128(smem_u32(sb) + kk * 32);
                tc::mma_bf16(tmem, da, db, idesc, (k0 > 0 || kk > 0) ? 1u : 0u);
            }
            tc::mma_commit(&bar);
        }
        const bool ok = mbar_wait_bounded(&bar, phase, kTcWait);
        phase ^= 1u;
        if (!ok) failed = 1;
        tc::fence_after_sync();
        __syncthreads();  // the tiles are free again
        if (failed) break;
    }
    if (!failed) {
        const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;
        const int row = m0 + 32 * (warp & 3) + lane;
        for (int c0 = 0; c0 < N; c0 += 16) {
            float v[16];
            tc::tmem_ld16(tmem + lane_base + (uint32_t)c0, v);
#pragma unroll
            for (int j = 0; j < 16; ++j) D[(size_t)row * N + c0 + j] = v[j];
        }
    } else if (tid == 0 && err) {
        atomicExch(err, 1);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_free(tmem, (uint32_t)ncols);
}

}  // namespace

cudaError_t launch_tc_gemm(const void *A, const void *B, float *D, int M, int N, int K, int *err, cudaStream_t s,
                           int64_t *launches) {
    if (M <= 0 || M % kTcM || K <= 0 || K % kTcK || N < 16 || N > 256 || N % 16) return cudaErrorInvalidValue;
    int ncols = 32;
    while (ncols < N) ncols <<= 1;
    const size_t smem = 1024 + (size_t)kTcM * kTcK * 2 + (size_t)N * kTcK * 2;
    // the attribute is the largest dynamic size any call uses (N = 256)
    const size_t smem_max = 1024 + (size_t)kTcM * kTcK * 2 + (size_t)256 * kTcK * 2;
    static KernelSetup ks;
    int per_sm = 0;
    cudaError_t e = ks.get(tc_gemm_kernel, 128, smem_max, true, &per_sm);
    if (e != cudaSuccess) return e;
    ++*launches;
    tc_gemm_kernel<<<M / kTcM, 128, smem, s>>>((const __nv_bfloat16 *)A, (const __nv_bfloat16 *)B, D, M, N, K,
                                                ncols, err);
    return cudaGetLastError();
}

}  // namespace msl
