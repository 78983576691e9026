// tc_probe.cu -- test-only library (built by tests/test_gpu_tc.py, never
// linked into libqmcgb.so): one CTA computes D = A * B^T (A 128 x K, B N x K,
// row-major BF16; D 128 x N, row-major FP32) through tcgen05.mma with the
// operand layout and descriptors of csrc/tc_sm100.cuh, so that the tests can
// compare it with an exact host product and pin the descriptor encodings
// every tensor-core kernel of the library relies on.  A completion wait that
// runs out sets bit 4 of *err (a device word the caller owns).
#include "../../qmctoolscl_gb300/csrc/tc_sm100.cuh"

namespace {

constexpr u32 WAIT_LIMIT = 1u << 22;  // mbarrier polls before giving up (a fraction of a second)

__global__ void __launch_bounds__(128) tc_probe_kernel(const __nv_bfloat16 *A, const __nv_bfloat16 *B, float *D,
                                                       u32 N, u32 K, u32 tcols, unsigned *err)
{
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ __align__(8) u64 bar;
    __shared__ u32 tmem_base;
    unsigned char *sA = sm, *sB = sm + 128 * K * 2;
    const u32 warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    if (warp == 0) tc::tmem_alloc(&tmem_base, tcols);
    for (u32 e = threadIdx.x; e < 128 * K; e += blockDim.x)
        *(__nv_bfloat16 *)(sA + tc::kmajor_offset(e / K, e % K, K)) = A[e];
    for (u32 e = threadIdx.x; e < N * K; e += blockDim.x)
        *(__nv_bfloat16 *)(sB + tc::kmajor_offset(e / K, e % K, K)) = B[e];
    tc::fence_smem_to_async();
    if (threadIdx.x == 0) tc::mbar_init(&bar, 1);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const u32 tmem = tmem_base;
    if (threadIdx.x == 0) {
        const u32 idesc = tc::idesc_bf16_f32(128, N);
        const u32 sbo = (K / 8) * 128;
        for (u32 s = 0; s < K / 16; s++)
            tc::mma_bf16(tmem, tc::smem_desc(sA + s * 256, 128, sbo), tc::smem_desc(sB + s * 256, 128, sbo), idesc,
                         s > 0);
        tc::mma_commit(&bar);
    }
    const bool ok = __all_sync(0xFFFFFFFFu, tc::mbar_wait(&bar, 0, WAIT_LIMIT));
    if (!ok && lane == 0) atomicOr(err, 4u);
    tc::fence_after_sync();
    if (ok) {
        const u32 row = warp * 32 + lane;
        for (u32 c0 = 0; c0 < N; c0 += 16) {
            u32 r[16];
            tc::tmem_ld16(tmem + ((warp * 32) << 16) + c0, r);
            tc::tmem_wait_ld();
#pragma unroll
            for (int j = 0; j < 16; j++) D[row * N + c0 + j] = __uint_as_float(r[j]);
        }
    } else {
        // give the MMAs one more bounded chance to finish before freeing their tensor memory
        tc::mbar_wait(&bar, 0, WAIT_LIMIT);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, tcols);
}

}  // namespace

// 0 on success, -1 for a shape outside the probe's range, -3 for a CUDA error.
extern "C" int tc_mma_probe(const void *A, const void *B, float *D, uint32_t N, uint32_t K, unsigned *err,
                            void *stream)
{
    if (!A || !B || !D || !err) return -1;
    if (N < 16 || N > 256 || N % 16 || K < 16 || K > 256 || K % 16) return -1;
    u32 tcols = 32;
    while (tcols < N) tcols <<= 1;
    const size_t smem = (size_t)(128 + N) * K * 2;
    if (cudaFuncSetAttribute(tc_probe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return -3;
    tc_probe_kernel<<<1, 128, smem, (cudaStream_t)stream>>>((const __nv_bfloat16 *)A, (const __nv_bfloat16 *)B, D,
                                                            N, K, tcols, err);
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}
