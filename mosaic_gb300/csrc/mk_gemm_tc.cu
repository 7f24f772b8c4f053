// General BF16 GEMM on the Blackwell tensor cores (tcgen05), FP32
// accumulation in tensor memory, with a fused epilogue:
//
//   C[row(m), n] = scale[m] * mask(m, n) * act( A[m, :] . B[:, n] (+ bias[n]) (+ C[m, n]) )
//
// A(m, k) at A[m*sam + k*sak], B(k, n) at B[k*sbk + n*sbn] (bf16, any
// strides: the same operand conventions as mk_gemm_bf16, so one kernel
// serves the MLP's forward pass, its input and weight gradients and the
// decoding of predicted frames). A CTA of 8 warps owns a 128 x BN tile of C:
// the K loop runs in chunks of 64 through MK_TCG_STAGES shared-memory
// stages, two chunks ahead of the tensor core: every thread stages part of
// a chunk into the K-major core-matrix layout of mk_tc.cuh (k-contiguous
// operands by asynchronous 16-byte cp.async copies, row-contiguous ones by
// batched 16-byte loads repacked in registers), one elected thread issues
// the chunk's four tcgen05.mma (K = 16 each) and commits them to the
// stage's mbarrier, which frees the stage for the chunk MK_TCG_STAGES
// later. The epilogue reads the accumulator back with tcgen05.ld (warp w:
// TMEM lanes 32 (w % 4) .. + 31 = tile rows, columns of half w / 4), one
// row per thread. Split-K over gridDim.z adds partial tiles into C with atomics.
// Every mbarrier wait is bounded; on expiry the CTA records
// MK_DEV_TIMEOUT_TMA, waits (bounded) for its issued MMAs, frees its TMEM
// and returns.
#include <cuda_bf16.h>

#include "mk_tc.cuh"

#define MK_TCG_BM 128
#define MK_TCG_BK 64
#define MK_TCG_STAGES 3
#define MK_TCG_NT 256

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
    int slices;                 // split-K slices per group (gridDim.z = groups * slices)
    long long gA, gB, gC, gCb, gbias, gmask;   // element strides between groups
};

// 16-byte asynchronous global -> shared copy; bytes beyond src_bytes are
// zero-filled (src_bytes 0: nothing is read).
__device__ __forceinline__ void mk_cp_async16(void *dst, const void *src, uint32_t src_bytes)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(mk_smem_addr(dst)), "l"(src),
                 "r"(src_bytes)
                 : "memory");
}
__device__ __forceinline__ void mk_cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void mk_cp_async_wait()
{
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Operand X(r, k) = X[r*sr + k*sk], rows [r0, r0 + R) x k [k0, k0 + 64) of
// a chunk (rows >= R_lim or k >= k_hi read as zero), into `dst` in the
// K-major core-matrix layout of an R x 64 tile (mk_umma_offset(r, k, 64)).
//
// k-contiguous operand (sk == 1, 16-byte aligned rows): asynchronous
// 16-byte copies, each one core-matrix row (8 consecutive k of one row).
// Thread e takes row 8 (e >> 6) + (e & 7) and k-vector (e >> 3) & 7: the 8
// threads of a group write 8 different core-matrix rows (all 32 banks), and
// a warp reads 64 contiguous bytes of each of 8 rows.
template <int R>
__device__ __forceinline__ void mk_tcg_issue_k(unsigned char *dst, const __nv_bfloat16 *X,
                                               long long sr, int r0, int R_lim, int k0, int k_hi)
{
#pragma unroll
    for (int i = 0; i < R * 8 / MK_TCG_NT; ++i) {
        const int e = threadIdx.x + i * MK_TCG_NT;
        const int r = ((e >> 6) << 3) + (e & 7), kv = (e >> 3) & 7;
        const int row = r0 + r, k = k0 + 8 * kv;
        const int valid = row < R_lim ? max(0, min(8, k_hi - k)) : 0;
        const __nv_bfloat16 *src = valid ? X + (long long)row * sr + k : X;
        mk_cp_async16(dst + mk_umma_offset(r, 8 * kv, MK_TCG_BK), src, (uint32_t)valid * 2u);
    }
}

// 8 consecutive rows of column k of a row-contiguous operand (zero outside).
__device__ __forceinline__ uint4 mk_tcg_load_rows8(const __nv_bfloat16 *X, long long sk, int row,
                                                   int R_lim, int k, int k_hi)
{
    if (k < k_hi && row + 8 <= R_lim)
        return *reinterpret_cast<const uint4 *>(X + (long long)k * sk + row);
    __nv_bfloat16 t[8];
    const __nv_bfloat16 zero = __float2bfloat16(0.f);
#pragma unroll
    for (int q = 0; q < 8; ++q) t[q] = (k < k_hi && row + q < R_lim) ? X[(long long)k * sk + row + q] : zero;
    return *reinterpret_cast<const uint4 *>(t);
}

// Row-contiguous operand (sr == 1, sk a multiple of 8, 16-byte aligned):
// every thread first loads all its 16-byte vectors (8 rows at k and at
// k + 1), then stores them as packed (k, k + 1) words.
template <int R>
__device__ __forceinline__ void mk_tcg_stage_r(unsigned char *dst, const __nv_bfloat16 *X,
                                               long long sk, int r0, int R_lim, int k0, int k_hi)
{
    constexpr int ITEMS = (R / 8) * 32 / MK_TCG_NT;
    uint4 va[ITEMS], vb[ITEMS];
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
        const int e = threadIdx.x + i * MK_TCG_NT;
        const int k = k0 + 2 * (e & 31), row = r0 + 8 * (e >> 5);
        va[i] = mk_tcg_load_rows8(X, sk, row, R_lim, k, k_hi);
        vb[i] = mk_tcg_load_rows8(X, sk, row, R_lim, k + 1, k_hi);
    }
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
        const int e = threadIdx.x + i * MK_TCG_NT;
        const int kp = e & 31, rg = e >> 5;
        const __nv_bfloat16 *a = reinterpret_cast<const __nv_bfloat16 *>(&va[i]);
        const __nv_bfloat16 *b = reinterpret_cast<const __nv_bfloat16 *>(&vb[i]);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            __nv_bfloat162 w;
            w.x = a[q];
            w.y = b[q];
            *reinterpret_cast<__nv_bfloat162 *>(dst + mk_umma_offset(8 * rg + q, 2 * kp, MK_TCG_BK)) = w;
        }
    }
}

// Any strides: element by element.
template <int R>
__device__ __forceinline__ void mk_tcg_stage_any(unsigned char *dst, const __nv_bfloat16 *X,
                                                 long long sr, long long sk, int r0, int R_lim,
                                                 int k0, int k_hi)
{
    const __nv_bfloat16 zero = __float2bfloat16(0.f);
    for (int e = threadIdx.x; e < R * MK_TCG_BK; e += MK_TCG_NT) {
        const int r = e / MK_TCG_BK, kk = e % MK_TCG_BK;
        const int row = r0 + r, k = k0 + kk;
        *reinterpret_cast<__nv_bfloat16 *>(dst + mk_umma_offset(r, kk, MK_TCG_BK)) =
            (row < R_lim && k < k_hi) ? X[(long long)row * sr + (long long)k * sk] : zero;
    }
}

// One operand's chunk by whichever path its layout allows (mode 0 async
// k-contiguous, 1 row-contiguous, 2 any).
template <int R>
__device__ __forceinline__ void mk_tcg_stage(unsigned char *dst, const __nv_bfloat16 *X, long long sr,
                                             long long sk, int r0, int R_lim, int k0, int k_hi,
                                             int mode)
{
    if (mode == 0)
        mk_tcg_issue_k<R>(dst, X, sr, r0, R_lim, k0, k_hi);
    else if (mode == 1)
        mk_tcg_stage_r<R>(dst, X, sk, r0, R_lim, k0, k_hi);
    else
        mk_tcg_stage_any<R>(dst, X, sr, sk, r0, R_lim, k0, k_hi);
}

// 16 consecutive floats p[0..15] (zero from index `avail` on); four 16-byte
// loads when `vec` and all 16 are there.
__device__ __forceinline__ void mk_tcg_load16(float (&d)[16], const float *p, int avail, bool vec)
{
    if (vec && avail >= 16) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float4 t = reinterpret_cast<const float4 *>(p)[q];
            d[4 * q] = t.x; d[4 * q + 1] = t.y; d[4 * q + 2] = t.z; d[4 * q + 3] = t.w;
        }
    } else {
#pragma unroll
        for (int j = 0; j < 16; ++j) d[j] = j < avail ? p[j] : 0.f;
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
    constexpr int S = MK_TCG_STAGES;
    constexpr int A_BYTES = MK_TCG_BM * MK_TCG_BK * 2;
    constexpr int STAGE_BYTES = A_BYTES + BN * MK_TCG_BK * 2;
    constexpr uint32_t NCOLS = BN < 32 ? 32u : (uint32_t)BN;
    constexpr uint32_t SBO = (MK_TCG_BK / 8) * 128;                 // between 8-row groups
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * MK_TCG_BM, n0 = blockIdx.x * BN;
    const int grp = blockIdx.z / g.slices, slice = blockIdx.z - grp * g.slices;
    const int k_lo = slice * g.k_per_slice;
    const int k_hi = min(g.K, k_lo + g.k_per_slice);
    const int nchunks = k_hi > k_lo ? (k_hi - k_lo + MK_TCG_BK - 1) / MK_TCG_BK : 0;
    // this CTA's group of the batched product
    g.A += grp * g.gA;
    g.B += grp * g.gB;
    if (g.C) g.C += grp * g.gC;
    if (g.Cb) g.Cb += grp * g.gCb;
    if (g.bias) g.bias += grp * g.gbias;
    if (g.mask) g.mask += grp * g.gmask;

    if (warp == 0) mk_tmem_alloc(tmem_slot, NCOLS);
    if (tid == 0) {
        for (int s = 0; s < S; ++s) mk_mbar_init(&bars[s], 1);
        mk_fence_barrier_init();
    }
    mk_tc_fence_before_sync();
    __syncthreads();
    mk_tc_fence_after_sync();
    const uint32_t tmem = *tmem_slot;

    const bool a_al = ((uintptr_t)g.A & 15) == 0, b_al = ((uintptr_t)g.B & 15) == 0;
    const int a_mode = (g.sak == 1 && (g.sam & 7) == 0 && a_al) ? 0
                       : (g.sam == 1 && (g.sak & 7) == 0 && a_al) ? 1 : 2;
    const int b_mode = (g.sbk == 1 && (g.sbn & 7) == 0 && b_al) ? 0
                       : (g.sbn == 1 && (g.sbk & 7) == 0 && b_al) ? 1 : 2;
    const uint32_t idesc = mk_umma_idesc_f16(MK_TCG_BM, BN, true);
    auto stage_chunk = [&](int c) {
        unsigned char *sa = stages + (c % S) * STAGE_BYTES;
        const int k0 = k_lo + c * MK_TCG_BK;
        mk_tcg_stage<MK_TCG_BM>(sa, g.A, g.sam, g.sak, m0, g.M, k0, k_hi, a_mode);
        mk_tcg_stage<BN>(sa + A_BYTES, g.B, g.sbn, g.sbk, n0, g.N, k0, k_hi, b_mode);
    };

    // Chunks 0 .. S-2 in flight before the first MMA; then, per chunk c,
    // chunk c + S - 1 is staged into the stage chunk c - 1 used (once its
    // MMAs are done) while chunk c's copies land and its MMAs run. One
    // cp.async group per chunk slot, empty ones included, so that
    // wait_group(S - 1) always means "chunk c has landed".
    bool ok = true;
    int last = -1;                                  // last chunk committed
#pragma unroll 1
    for (int c = 0; c < S - 1; ++c) {
        if (c < nchunks) stage_chunk(c);
        mk_cp_async_commit();
    }
#pragma unroll 1
    for (int c = 0; c < nchunks; ++c) {
        const int cn = c + S - 1;
        if (cn < nchunks) {
            if (c >= 1) {
                const bool w = mk_mbar_wait_bounded(&bars[(c - 1) % S], ((c - 1) / S) & 1,
                                                    MK_WAIT_LIMIT_NS / 4);
                if (__syncthreads_or(!w)) {
                    ok = false;
                    break;
                }
            }
            stage_chunk(cn);
        }
        mk_cp_async_commit();
        mk_cp_async_wait<S - 1>();
        mk_fence_proxy_async();          // copies and stores -> visible to the tensor core
        mk_tc_fence_before_sync();
        __syncthreads();
        if (tid == 0) {
            mk_tc_fence_after_sync();
            const uint32_t a0 = mk_smem_addr(stages + (c % S) * STAGE_BYTES);
            const uint32_t b0 = a0 + A_BYTES;
#pragma unroll
            for (int kk = 0; kk < MK_TCG_BK / 16; ++kk)
                mk_umma_f16(tmem, mk_umma_sdesc(a0 + 256u * kk, 128u, SBO),
                            mk_umma_sdesc(b0 + 256u * kk, 128u, SBO), idesc,
                            (c > 0 || kk > 0) ? 1u : 0u);
            mk_umma_commit(&bars[c % S]);
        }
        last = c;
    }
    mk_cp_async_wait<0>();
    if (last >= 0) {
        // the last commit completes after every MMA issued before it
        const bool w = mk_mbar_wait_bounded(&bars[last % S], (last / S) & 1, MK_WAIT_LIMIT_NS / 4);
        ok = ok && w;
    }
    mk_tc_fence_after_sync();
    if (__syncthreads_or(!ok)) {
        if (tid == 0) atomicExch(status, MK_DEV_TIMEOUT_TMA);
    } else {
        // Epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (the lane
        // quarter a warp may access) for half w / 4 of the columns; thread =
        // one row of the tile, 16 columns per TMEM load; every operand of a
        // 16-column group is loaded before any store.
        const int quarter = warp & 3, half = warp >> 2;
        const int m = m0 + 32 * quarter + lane;
        const bool row_ok = m < g.M;
        const long long orow = row_ok ? (g.row_map ? g.row_map[m] : (long long)m) : 0;
        const float rs = (row_ok && g.row_scale) ? g.row_scale[m] : 1.f;
        const bool split = g.slices > 1;
        const bool c_vec = g.C && ((uintptr_t)g.C & 15) == 0 && (g.ldc & 3) == 0;
        const bool b_vec = g.bias && ((uintptr_t)g.bias & 15) == 0;
        const bool m_vec = g.mask && ((uintptr_t)g.mask & 15) == 0 && (g.ldm & 3) == 0;
        const bool cb_vec = g.Cb && ((uintptr_t)g.Cb & 15) == 0 && (g.ldcb & 7) == 0;
#pragma unroll 1
        for (int c0 = half * (BN / 2); c0 < (half + 1) * (BN / 2); c0 += 16) {
            float v[16];
            if (nchunks > 0) {
                mk_tmem_ld16(tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)c0, v);
            } else {
#pragma unroll
                for (int j = 0; j < 16; ++j) v[j] = 0.f;
            }
            const int nb = n0 + c0;
            const int avail = min(16, g.N - nb);
            if (!row_ok || avail <= 0) continue;
            if (split) {
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    if (j < avail) atomicAdd(&g.C[(long long)m * g.ldc + nb + j], v[j]);
                continue;
            }
            float t[16];
            if (g.flags & MK_GEMM_BIAS) {
                mk_tcg_load16(t, g.bias + nb, avail, b_vec);
#pragma unroll
                for (int j = 0; j < 16; ++j) v[j] += t[j];
            }
            if (g.flags & MK_GEMM_ACCUMULATE) {
                mk_tcg_load16(t, g.C + (long long)m * g.ldc + nb, avail, c_vec);
#pragma unroll
                for (int j = 0; j < 16; ++j) v[j] += t[j];
            }
            if (g.flags & MK_GEMM_RELU) {
#pragma unroll
                for (int j = 0; j < 16; ++j) v[j] = fmaxf(v[j], 0.f);
            }
            if (g.mask) {
                mk_tcg_load16(t, g.mask + (long long)m * g.ldm + nb, avail, m_vec);
#pragma unroll
                for (int j = 0; j < 16; ++j) v[j] = t[j] > 0.f ? v[j] : 0.f;
            }
#pragma unroll
            for (int j = 0; j < 16; ++j) v[j] *= rs;
            if (g.C) {
                float *o = g.C + orow * g.ldc + nb;
                if (c_vec && avail == 16) {
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        reinterpret_cast<float4 *>(o)[q] =
                            make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                } else {
#pragma unroll
                    for (int j = 0; j < 16; ++j)
                        if (j < avail) o[j] = v[j];
                }
            }
            if (g.Cb) {
                __nv_bfloat16 *o = g.Cb + orow * g.ldcb + nb;
                if (cb_vec && avail == 16) {
                    __nv_bfloat162 h[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) h[q] = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);
                    reinterpret_cast<uint4 *>(o)[0] = reinterpret_cast<const uint4 *>(h)[0];
                    reinterpret_cast<uint4 *>(o)[1] = reinterpret_cast<const uint4 *>(h)[1];
                } else {
#pragma unroll
                    for (int j = 0; j < 16; ++j)
                        if (j < avail) o[j] = __float2bfloat16(v[j]);
                }
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

extern "C" int mk_gemm_tc_groups(int groups, const long long *group_strides, int M, int N, int K,
                                 const void *A, long long sam, long long sak, const void *B,
                                 long long sbk, long long sbn, float *C, long long ldc,
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
    MK_REQUIRE(groups >= 1 && groups <= 1024, "mk_gemm_tc: groups must be in [1, 1024]");
    long long gs[6] = {0, 0, 0, 0, 0, 0};
    if (groups > 1) {
        MK_REQUIRE(group_strides, "mk_gemm_tc: group strides needed for groups > 1");
        for (int i = 0; i < 6; ++i) gs[i] = group_strides[i];
        MK_REQUIRE((!C || gs[2] != 0) && (!Cb || gs[3] != 0),
                   "mk_gemm_tc: groups must write to different outputs");
        MK_REQUIRE(!row_scale && !row_map, "mk_gemm_tc: row_scale / row_map need groups == 1");
    }
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
    g.gA = gs[0]; g.gB = gs[1]; g.gC = gs[2]; g.gCb = gs[3]; g.gbias = gs[4]; g.gmask = gs[5];
    g.k_per_slice = (K + MK_TCG_BK - 1) / MK_TCG_BK * MK_TCG_BK;
    g.slices = 1;
    // Few output tiles and a long K (the weight gradients: K = batch):
    // split K over up to 8 slices that add into C, when the epilogue is a
    // plain store or accumulate into C.
    const int tiles = (int)(grid.x * grid.y) * groups;
    if (tiles < 64 && K >= 4 * MK_TCG_BK && C && !Cb && !relu_mask && !row_scale && !row_map &&
        !(flags & (MK_GEMM_BIAS | MK_GEMM_RELU))) {
        const int chunks = (K + MK_TCG_BK - 1) / MK_TCG_BK;
        int z = std::min(8, std::min(chunks / 2, (128 + tiles - 1) / tiles));
        if (z > 1) {
            const int per = (chunks + z - 1) / z;
            g.k_per_slice = per * MK_TCG_BK;
            g.slices = (chunks + per - 1) / per;        // every slice non-empty
            if (!(flags & MK_GEMM_ACCUMULATE))
                for (int q = 0; q < groups; ++q)
                    MK_CHECK_CUDA(cudaMemset2DAsync(C + q * gs[2], sizeof(float) * (size_t)ldc, 0,
                                                    sizeof(float) * (size_t)N, (size_t)M, st));
        }
    }
    MK_REQUIRE((long long)groups * g.slices < 65536, "mk_gemm_tc: too many groups");
    grid.z = (unsigned)(groups * g.slices);
    return bn == 128 ? mk_tcg_launch<128>(g, grid, st, status) : mk_tcg_launch<64>(g, grid, st, status);
}

extern "C" int mk_gemm_tc(int M, int N, int K, const void *A, long long sam, long long sak,
                          const void *B, long long sbk, long long sbn, float *C, long long ldc,
                          const float *bias, int flags, void *Cb, long long ldcb,
                          const float *relu_mask, long long ldm, const float *row_scale,
                          const long long *row_map, void *stream)
{
    return mk_gemm_tc_groups(1, nullptr, M, N, K, A, sam, sak, B, sbk, sbn, C, ldc, bias, flags, Cb,
                             ldcb, relu_mask, ldm, row_scale, row_map, stream);
}
