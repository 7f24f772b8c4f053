// A single-tile tensor-core product on tcgen05: C (128 x N, FP32) =
// A (128 x K) . B (N x K)^T, FP16 or BF16 operands, accumulated in TMEM.
// It exercises the descriptors and the TMEM round trip of mk_tc.cuh in
// isolation -- the self-check of the tensor-core path the library's other
// tcgen05 kernels build on.
#include "mk_tc.cuh"

#define MK_TC_NT 128
#define MK_TC_MAXK 128
#define MK_TC_MAXN 256

__global__ void __launch_bounds__(MK_TC_NT)
    mk_tc_gemm_kernel(int N, int K, int bf16, const uint16_t *__restrict__ A,
                      const uint16_t *__restrict__ B, float *__restrict__ C, int *status)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + 8);
    unsigned char *sa = smem + 1024;                          // 128 x K
    unsigned char *sb = sa + (size_t)128 * K * 2;             // N x K
    const int tid = threadIdx.x, warp = tid >> 5;
    // TMEM columns: the accumulator's N, rounded up to a power of two >= 32
    uint32_t ncols = 32;
    while (ncols < (uint32_t)N) ncols <<= 1;
    if (warp == 0) mk_tmem_alloc(tmem_slot, ncols);
    if (tid == 0) {
        mk_mbar_init(bar, 1);
        mk_fence_barrier_init();
    }
    // operands into the K-major core-matrix layout
    for (int e = tid; e < 128 * K; e += MK_TC_NT) {
        const int r = e / K, k = e - r * K;
        *reinterpret_cast<uint16_t *>(sa + mk_umma_offset(r, k, K)) = A[e];
    }
    for (int e = tid; e < N * K; e += MK_TC_NT) {
        const int r = e / K, k = e - r * K;
        *reinterpret_cast<uint16_t *>(sb + mk_umma_offset(r, k, K)) = B[e];
    }
    mk_fence_proxy_async();           // generic-proxy writes -> visible to the tensor core
    mk_tc_fence_before_sync();
    __syncthreads();
    mk_tc_fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    if (tid == 0) {
        const uint32_t idesc = mk_umma_idesc_f16(128, N, bf16 != 0);
        const uint32_t a0 = mk_smem_addr(sa), b0 = mk_smem_addr(sb);
        const uint32_t sbo = (uint32_t)(K >> 3) << 7;
        for (int kk = 0; kk < K / 16; ++kk) {
            const uint64_t ad = mk_umma_sdesc(a0 + 256u * kk, 128u, sbo);
            const uint64_t bd = mk_umma_sdesc(b0 + 256u * kk, 128u, sbo);
            mk_umma_f16(tmem, ad, bd, idesc, kk > 0 ? 1u : 0u);
        }
        mk_umma_commit(bar);
    }
    const bool ok = mk_mbar_wait_bounded(bar, 0, MK_WAIT_LIMIT_NS / 4);
    mk_tc_fence_after_sync();
    if (__syncthreads_or(!ok)) {
        if (tid == 0) atomicExch(status, MK_DEV_TIMEOUT_TMA);
    } else {
        // warp w reads TMEM lanes 32w .. 32w + 31 = rows of C
        const int row = 32 * warp + (tid & 31);
        for (int c = 0; c < N; c += 16) {
            float v[16];
            mk_tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c, v);
#pragma unroll
            for (int j = 0; j < 16; ++j) C[(size_t)row * N + c + j] = v[j];
        }
    }
    mk_tc_fence_before_sync();
    __syncthreads();
    if (warp == 0) mk_tmem_dealloc(tmem, ncols);
}

static __device__ int g_tc_status;

static int mk_tc_read_status(cudaStream_t st)
{
    int v = 0, zero = 0;
    if (cudaMemcpyFromSymbolAsync(&v, g_tc_status, sizeof(int), 0, cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaMemcpyToSymbolAsync(g_tc_status, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        mk_set_error("mk_sync_status: cannot read the tensor-core status word");
        return MK_ECUDA;
    }
    if (v == MK_DEV_TIMEOUT_TMA) {
        mk_set_error("tensor-core product: the MMA did not complete within its time limit");
        return MK_ETIMEOUT;
    }
    return MK_OK;
}

extern "C" int mk_tc_gemm(int N, int K, int bf16, const void *A, const void *B, float *C,
                          void *stream)
{
    MK_REQUIRE(A && B && C, "mk_tc_gemm: null argument");
    MK_REQUIRE(N >= 16 && N <= MK_TC_MAXN && N % 16 == 0,
               "mk_tc_gemm: N must be a multiple of 16 in [16, %d]", MK_TC_MAXN);
    MK_REQUIRE(K >= 16 && K <= MK_TC_MAXK && K % 16 == 0,
               "mk_tc_gemm: K must be a multiple of 16 in [16, %d]", MK_TC_MAXK);
    mk_register_status_reader(mk_tc_read_status);
    int *status = nullptr;
    MK_CHECK_CUDA(cudaGetSymbolAddress((void **)&status, g_tc_status));
    const size_t smem = 1024 + (size_t)(128 + N) * K * 2;
    MK_CHECK_CUDA(cudaFuncSetAttribute((const void *)mk_tc_gemm_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    mk_tc_gemm_kernel<<<1, MK_TC_NT, smem, mk_stream(stream)>>>(
        N, K, bf16, static_cast<const uint16_t *>(A), static_cast<const uint16_t *>(B), C, status);
    MK_CHECK_CUDA(cudaGetLastError());
    return MK_OK;
}
