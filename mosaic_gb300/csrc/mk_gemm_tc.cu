// General BF16 GEMM on the Blackwell tensor cores (tcgen05), FP32
// accumulation in tensor memory, with a fused epilogue:
//
//   C[row(m), n] = scale[m] * mask(m, n) * act( A[m, :] . B[:, n] (+ bias[n]) (+ C[m, n]) )
//
// A(m, k) at A[m*sam + k*sak], B(k, n) at B[k*sbk + n*sbn] (bf16, any
// strides: the same operand conventions as mk_gemm_bf16, so one kernel
// serves the MLP's forward pass, its input and weight gradients and the
// decoding of predicted frames). A CTA of 4 warps owns a 128 x BN tile of C:
// the K loop runs in chunks of 64 through MK_TCG_STAGES shared-memory
// stages; every thread stages part of a chunk (16-byte loads along whichever
// of k or m/n the operand is contiguous in) into the K-major core-matrix
// layout of mk_tc.cuh, one elected thread issues the chunk's four
// tcgen05.mma (K = 16 each) and commits them to the stage's mbarrier, which
// frees the stage for the chunk MK_TCG_STAGES later, so staging overlaps
// the tensor core. The epilogue reads the accumulator back with
// tcgen05.ld (warp w: TMEM lanes 32w..32w+31 = tile rows), one row per
// thread. Split-K over gridDim.z adds partial tiles into C with atomics.
// Every mbarrier wait is bounded; on expiry the CTA records
// MK_DEV_TIMEOUT_TMA, waits (bounded) for its issued MMAs, frees its TMEM
// and returns.
#include <cuda_bf16.h>

#include "mk_tc.cuh"

#define MK_TCG_BM 128
#define MK_TCG_BK 64
#define MK_TCG_STAGES 3
#define MK_TCG_NT 128

#define MK_GEMM_ACCUMULATE 1
#define MK_GEMM_BIAS 2
#define MK_GEMM_RELU 4

struct MkTcGemm {
    int M, N, K, k_per_slice, flags;
    const __nv_bfloat16 *A;
    long long sam, sak;
    const __nv_bfloat16 *B;
    long long sbk, sbn;
    float *C;
    long long ldc;
    const float *bias;
    __nv_bfloat16 *Cb;
    long long ldcb;
    const float *mask;          // relu mask: zero where mask[m*ldm + n] <= 0
    long long ldm;
    const float *row_scale;     // multiplies row m
    const long long *row_map;   // output row of row m
};

// Stage rows [r0, r0 + R) x k [k0, k0 + 64) of an operand X(r, k) =
// X[r*sr + k*sk] (rows >= R_lim or k >= k_hi read as zero) into `dst` in the
// K-major core-matrix layout of a R x 64 tile (mk_umma_offset(r, k, 64)).
template <int R>
__device__ __forceinline__ void mk_tcg_stage(unsigned char *dst, const __nv_bfloat16 *X,
                                             long long sr, long long sk, int r0, int R_lim,
                                             int k0, int k_hi, bool k_vec, bool r_vec)
{
    const int tid = threadIdx.x;
    const __nv_bfloat16 zero = __float2bfloat16(0.f);
    if (k_vec) {
        // 8 consecutive k of one row per 16-byte load; contiguous 16-byte stores
        for (int e = tid; e < R * 8; e += MK_TCG_NT) {
            const int r = e >> 3, kv = e & 7;
            const int row = r0 + r, k = k0 + 8 * kv;
            uint4 v;
            if (row < R_lim && k + 8 <= k_hi) {
                v = *reinterpret_cast<const uint4 *>(X + (long long)row * sr + k);
            } else {
                __nv_bfloat16 t[8];
#pragma unroll
                for (int q = 0; q < 8; ++q)
                    t[q] = (row < R_lim && k + q < k_hi) ? X[(long long)row * sr + k + q] : zero;
                v = *reinterpret_cast<const uint4 *>(t);
            }
            *reinterpret_cast<uint4 *>(dst + mk_umma_offset(r, 8 * kv, MK_TCG_BK)) = v;
        }
    } else if (r_vec) {
        // 8 consecutive rows at k and at k + 1 per thread (two 16-byte
        // loads), stored as 8 packed (k, k + 1) words
        for (int e = tid; e < (R / 8) * 32; e += MK_TCG_NT) {
            const int kp = e & 31, rg = e >> 5;
            const int k = k0 + 2 * kp, row = r0 + 8 * rg;
            __nv_bfloat16 a[8], b[8];
            if (row + 8 <= R_lim && k + 2 <= k_hi) {
                *reinterpret_cast<uint4 *>(a) = *reinterpret_cast<const uint4 *>(X + (long long)k * sk + row);
                *reinterpret_cast<uint4 *>(b) =
                    *reinterpret_cast<const uint4 *>(X + (long long)(k + 1) * sk + row);
            } else {
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    a[q] = (row + q < R_lim && k < k_hi) ? X[(long long)k * sk + row + q] : zero;
                    b[q] = (row + q < R_lim && k + 1 < k_hi) ? X[(long long)(k + 1) * sk + row + q]
                                                             : zero;
                }
            }
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                __nv_bfloat162 w;
                w.x = a[q];
                w.y = b[q];
                *reinterpret_cast<__nv_bfloat162 *>(dst + mk_umma_offset(8 * rg + q, 2 * kp, MK_TCG_BK)) = w;
            }
        }
    } else {
        for (int e = tid; e < R * MK_TCG_BK; e += MK_TCG_NT) {
            const int r = e / MK_TCG_BK, kk = e % MK_TCG_BK;
            const int row = r0 + r, k = k0 + kk;
            *reinterpret_cast<__nv_bfloat16 *>(dst + mk_umma_offset(r, kk, MK_TCG_BK)) =
                (row < R_lim && k < k_hi) ? X[(long long)row * sr + (long long)k * sk] : zero;
        }
    }
}

template <int BN>
__global__ void __launch_bounds__(MK_TCG_NT) mk_gemm_tc_kernel(MkTcGemm g, int *status)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // 1024-byte aligned base for the operand stages
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem);            // MK_TCG_STAGES barriers
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + 64);
    unsigned char *stages = smem + 1024;
    constexpr int A_BYTES = MK_TCG_BM * MK_TCG_BK * 2;
    constexpr int STAGE_BYTES = A_BYTES + BN * MK_TCG_BK * 2;
    constexpr uint32_t NCOLS = BN < 32 ? 32u : (uint32_t)BN;
    constexpr uint32_t SBO = (MK_TCG_BK / 8) * 128;                 // between 8-row groups
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * MK_TCG_BM, n0 = blockIdx.x * BN;
    const int k_lo = blockIdx.z * g.k_per_slice;
    const int k_hi = min(g.K, k_lo + g.k_per_slice);
    const int nchunks = k_hi > k_lo ? (k_hi - k_lo + MK_TCG_BK - 1) / MK_TCG_BK : 0;

    if (warp == 0) mk_tmem_alloc(tmem_slot, NCOLS);
    if (tid == 0) {
        for (int s = 0; s < MK_TCG_STAGES; ++s) mk_mbar_init(&bars[s], 1);
        mk_fence_barrier_init();
    }
    mk_tc_fence_before_sync();
    __syncthreads();
    mk_tc_fence_after_sync();
    const uint32_t tmem = *tmem_slot;

    const bool a_k = g.sak == 1 && (g.sam & 7) == 0 && ((uintptr_t)g.A & 15) == 0;
    const bool a_r = !a_k && g.sam == 1 && (g.sak & 7) == 0 && ((uintptr_t)g.A & 15) == 0;
    const bool b_k = g.sbk == 1 && (g.sbn & 7) == 0 && ((uintptr_t)g.B & 15) == 0;
    const bool b_r = !b_k && g.sbn == 1 && (g.sbk & 7) == 0 && ((uintptr_t)g.B & 15) == 0;
    const uint32_t idesc = mk_umma_idesc_f16(MK_TCG_BM, BN, true);

    bool ok = true;
    int last = -1;                                  // last chunk committed
    for (int c = 0; c < nchunks; ++c) {
        const int s = c % MK_TCG_STAGES;
        if (c >= MK_TCG_STAGES) {
            // the chunk MK_TCG_STAGES back used this stage: wait for its MMAs
            const bool w = mk_mbar_wait_bounded(&bars[s], ((c - MK_TCG_STAGES) / MK_TCG_STAGES) & 1,
                                                MK_WAIT_LIMIT_NS / 4);
            if (__syncthreads_or(!w)) {
                ok = false;
                break;
            }
        }
        unsigned char *sa = stages + s * STAGE_BYTES;
        unsigned char *sb = sa + A_BYTES;
        const int k0 = k_lo + c * MK_TCG_BK;
        mk_tcg_stage<MK_TCG_BM>(sa, g.A, g.sam, g.sak, m0, g.M, k0, k_hi, a_k, a_r);
        mk_tcg_stage<BN>(sb, g.B, g.sbn, g.sbk, n0, g.N, k0, k_hi, b_k, b_r);
        mk_fence_proxy_async();          // generic-proxy stores -> visible to the tensor core
        mk_tc_fence_before_sync();
        __syncthreads();
        if (tid == 0) {
            mk_tc_fence_after_sync();
            const uint32_t a0 = mk_smem_addr(sa), b0 = mk_smem_addr(sb);
#pragma unroll
            for (int kk = 0; kk < MK_TCG_BK / 16; ++kk)
                mk_umma_f16(tmem, mk_umma_sdesc(a0 + 256u * kk, 128u, SBO),
                            mk_umma_sdesc(b0 + 256u * kk, 128u, SBO), idesc,
                            (c > 0 || kk > 0) ? 1u : 0u);
            mk_umma_commit(&bars[s]);
        }
        last = c;
    }
    if (last >= 0) {
        // the last commit completes after every MMA issued before it
        const bool w = mk_mbar_wait_bounded(&bars[last % MK_TCG_STAGES], (last / MK_TCG_STAGES) & 1,
                                            MK_WAIT_LIMIT_NS / 4);
        ok = ok && w;
    }
    mk_tc_fence_after_sync();
    if (__syncthreads_or(!ok)) {
        if (tid == 0) atomicExch(status, MK_DEV_TIMEOUT_TMA);
    } else {
        const int m = m0 + 32 * warp + lane;
        const bool row_ok = m < g.M;
        const long long orow = row_ok ? (g.row_map ? g.row_map[m] : (long long)m) : 0;
        const float rs = (row_ok && g.row_scale) ? g.row_scale[m] : 1.f;
        const bool split = gridDim.z > 1;
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 16) {
            float v[16];
            if (nchunks > 0) {
                mk_tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, v);
            } else {
#pragma unroll
                for (int j = 0; j < 16; ++j) v[j] = 0.f;
            }
            if (!row_ok) continue;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int n = n0 + c0 + j;
                if (n >= g.N) break;
                float x = v[j];
                if (split) {
                    atomicAdd(&g.C[(long long)m * g.ldc + n], x);
                    continue;
                }
                if (g.flags & MK_GEMM_BIAS) x += g.bias[n];
                if (g.flags & MK_GEMM_ACCUMULATE) x += g.C[(long long)m * g.ldc + n];
                if (g.flags & MK_GEMM_RELU) x = fmaxf(x, 0.f);
                if (g.mask && !(g.mask[(long long)m * g.ldm + n] > 0.f)) x = 0.f;
                x *= rs;
                if (g.C) g.C[orow * g.ldc + n] = x;
                if (g.Cb) g.Cb[orow * g.ldcb + n] = __float2bfloat16(x);
            }
        }
    }
    mk_tc_fence_before_sync();
    __syncthreads();
    if (warp == 0) mk_tmem_dealloc(tmem, NCOLS);
}

static __device__ int g_tcg_status;

static int mk_tcg_read_status(cudaStream_t st)
{
    int v = 0, zero = 0;
    if (cudaMemcpyFromSymbolAsync(&v, g_tcg_status, sizeof(int), 0, cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaMemcpyToSymbolAsync(g_tcg_status, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        mk_set_error("mk_sync_status: cannot read the tensor-core GEMM status word");
        return MK_ECUDA;
    }
    if (v == MK_DEV_TIMEOUT_TMA) {
        mk_set_error("tensor-core GEMM: an MMA did not complete within its time limit");
        return MK_ETIMEOUT;
    }
    return MK_OK;
}

template <int BN>
static int mk_tcg_launch(const MkTcGemm &g, dim3 grid, cudaStream_t st, int *status)
{
    const size_t smem = 2048 + (size_t)MK_TCG_STAGES * (MK_TCG_BM + BN) * MK_TCG_BK * 2;
    MK_CHECK_CUDA(cudaFuncSetAttribute((const void *)mk_gemm_tc_kernel<BN>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    mk_gemm_tc_kernel<BN><<<grid, MK_TCG_NT, smem, st>>>(g, status);
    MK_CHECK_CUDA(cudaGetLastError());
    return MK_OK;
}

extern "C" int mk_gemm_tc(int M, int N, int K, const void *A, long long sam, long long sak,
                          const void *B, long long sbk, long long sbn, float *C, long long ldc,
                          const float *bias, int flags, void *Cb, long long ldcb,
                          const float *relu_mask, long long ldm, const float *row_scale,
                          const long long *row_map, void *stream)
{
    MK_REQUIRE(M > 0 && N > 0 && K > 0 && A && B, "mk_gemm_tc: bad shape or null operand");
    MK_REQUIRE(C || Cb, "mk_gemm_tc: no output");
    MK_REQUIRE(!(flags & MK_GEMM_ACCUMULATE) || C, "mk_gemm_tc: accumulate needs C");
    MK_REQUIRE(!(flags & MK_GEMM_BIAS) || bias, "mk_gemm_tc: bias flag without bias");
    MK_REQUIRE(!(flags & MK_GEMM_ACCUMULATE) || !row_map,
               "mk_gemm_tc: accumulate reads row m of C; it cannot be combined with row_map");
    MK_REQUIRE(!relu_mask || ldm >= N, "mk_gemm_tc: mask row stride below N");
    cudaStream_t st = mk_stream(stream);
    mk_register_status_reader(mk_tcg_read_status);
    int *status = nullptr;
    MK_CHECK_CUDA(cudaGetSymbolAddress((void **)&status, g_tcg_status));
    // 128-column tiles for wide outputs, 64 otherwise (more CTAs on the
    // MLP's 256-wide layers)
    const int bn = N >= 2048 ? 128 : 64;
    dim3 grid((N + bn - 1) / bn, (M + MK_TCG_BM - 1) / MK_TCG_BM, 1);
    MK_REQUIRE(grid.y < 65536, "mk_gemm_tc: M too large");
    MkTcGemm g{};
    g.M = M; g.N = N; g.K = K; g.flags = flags;
    g.A = static_cast<const __nv_bfloat16 *>(A); g.sam = sam; g.sak = sak;
    g.B = static_cast<const __nv_bfloat16 *>(B); g.sbk = sbk; g.sbn = sbn;
    g.C = C; g.ldc = ldc; g.bias = bias;
    g.Cb = static_cast<__nv_bfloat16 *>(Cb); g.ldcb = ldcb;
    g.mask = relu_mask; g.ldm = ldm; g.row_scale = row_scale; g.row_map = row_map;
    g.k_per_slice = (K + MK_TCG_BK - 1) / MK_TCG_BK * MK_TCG_BK;
    // Few output tiles and a long K (the weight gradients: K = batch):
    // split K over up to 8 slices that add into C, when the epilogue is a
    // plain store or accumulate into C.
    const int tiles = (int)(grid.x * grid.y);
    if (tiles < 64 && K >= 4 * MK_TCG_BK && C && !Cb && !relu_mask && !row_scale && !row_map &&
        !(flags & (MK_GEMM_BIAS | MK_GEMM_RELU))) {
        const int chunks = (K + MK_TCG_BK - 1) / MK_TCG_BK;
        int z = std::min(8, std::min(chunks / 2, (128 + tiles - 1) / tiles));
        if (z > 1) {
            const int per = (chunks + z - 1) / z;
            g.k_per_slice = per * MK_TCG_BK;
            z = (chunks + per - 1) / per;               // every slice non-empty
            grid.z = (unsigned)z;
            if (!(flags & MK_GEMM_ACCUMULATE))
                MK_CHECK_CUDA(cudaMemset2DAsync(C, sizeof(float) * (size_t)ldc, 0,
                                                sizeof(float) * (size_t)N, (size_t)M, st));
        }
    }
    return bn == 128 ? mk_tcg_launch<128>(g, grid, st, status) : mk_tcg_launch<64>(g, grid, st, status);
}
