// BF16 multilayer perceptron kernels for the scan surrogate: GEMM with FP32
// accumulation (tensor cores through mma.sync m16n8k16), Fourier features,
// ReLU backward, bias gradient, MSE loss and Adam with FP32 master weights.
//
// GEMM: C[M, N] (+)= A[M, K] B[K, N] (+ bias[n]) (ReLU), A and B given by
// element strides, so one kernel serves the forward pass (X W^T), the input
// gradient (dY W) and the weight gradient (dY^T X). Tiles of 64 x 64 x 32
// staged in shared memory with k contiguous (A as [m][k], B as [n][k]);
// 4 warps, each 32 x 32 = 2 x 4 mma tiles. Out-of-range rows/columns/k read
// as zero and are never written.
#include <cuda_bf16.h>

#include "mk_common.cuh"

#define MLP_BM 64
#define MLP_BN 64
#define MLP_BK 32
#define MLP_PAD 8      // bf16 elements of padding per smem row (bank spread)

#define MK_GEMM_ACCUMULATE 1
#define MK_GEMM_BIAS 2
#define MK_GEMM_RELU 4

__device__ __forceinline__ void mk_mma_bf16(float (&d)[4], const uint32_t (&a)[4],
                                            const uint32_t (&b)[2])
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__global__ void __launch_bounds__(128) mk_gemm_bf16_kernel(
    int M, int N, int K, const __nv_bfloat16 *__restrict__ A, long long sam, long long sak,
    const __nv_bfloat16 *__restrict__ B, long long sbk, long long sbn, float *__restrict__ C,
    long long ldc, const float *__restrict__ bias, int flags, __nv_bfloat16 *__restrict__ Cb,
    long long ldcb)
{
    __shared__ __align__(16) __nv_bfloat16 As[MLP_BM][MLP_BK + MLP_PAD];
    __shared__ __align__(16) __nv_bfloat16 Bs[MLP_BN][MLP_BK + MLP_PAD];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * MLP_BM, n0 = blockIdx.x * MLP_BN;
    // split-K: slice blockIdx.z of gridDim.z sums k in [k_lo, k_hi) and adds
    // its partial product into C (which the host has zeroed or holds the
    // accumulation base); one slice: the whole K and the full epilogue
    const int kper = ((K + gridDim.z - 1) / gridDim.z + MLP_BK - 1) / MLP_BK * MLP_BK;
    const int k_lo = blockIdx.z * kper, k_hi = min(K, k_lo + kper);
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;   // warp sub-tile
    const int g = lane >> 2, t4 = lane & 3;                   // mma group / thread in group
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;

    const __nv_bfloat16 zero = __float2bfloat16(0.f);
    // operands contiguous in k (the forward pass): 8 bf16 per 16-byte load
    const bool a_vec = sak == 1 && (sam & 7) == 0 && ((uintptr_t)A & 15) == 0;
    const bool b_vec = sbk == 1 && (sbn & 7) == 0 && ((uintptr_t)B & 15) == 0;
    for (int k0 = k_lo; k0 < k_hi; k0 += MLP_BK) {
        if (a_vec) {
            for (int e = tid; e < MLP_BM * MLP_BK / 8; e += 128) {
                const int r = e / (MLP_BK / 8), c = (e % (MLP_BK / 8)) * 8;
                const int m = m0 + r, k = k0 + c;
                if (m < M && k + 7 < k_hi) {
                    *reinterpret_cast<uint4 *>(&As[r][c]) =
                        *reinterpret_cast<const uint4 *>(A + (long long)m * sam + k);
                } else {
#pragma unroll
                    for (int q = 0; q < 8; ++q)
                        As[r][c + q] = (m < M && k + q < k_hi) ? A[(long long)m * sam + k + q] : zero;
                }
            }
        } else {
            for (int e = tid; e < MLP_BM * MLP_BK; e += 128) {
                const int r = e / MLP_BK, c = e % MLP_BK;
                const int m = m0 + r, k = k0 + c;
                As[r][c] = (m < M && k < k_hi) ? A[(long long)m * sam + (long long)k * sak] : zero;
            }
        }
        if (b_vec) {
            for (int e = tid; e < MLP_BN * MLP_BK / 8; e += 128) {
                const int r = e / (MLP_BK / 8), c = (e % (MLP_BK / 8)) * 8;
                const int n = n0 + r, k = k0 + c;
                if (n < N && k + 7 < k_hi) {
                    *reinterpret_cast<uint4 *>(&Bs[r][c]) =
                        *reinterpret_cast<const uint4 *>(B + (long long)n * sbn + k);
                } else {
#pragma unroll
                    for (int q = 0; q < 8; ++q)
                        Bs[r][c + q] = (n < N && k + q < k_hi) ? B[(long long)n * sbn + k + q] : zero;
                }
            }
        } else {
            for (int e = tid; e < MLP_BN * MLP_BK; e += 128) {
                const int r = e / MLP_BK, c = e % MLP_BK;
                const int n = n0 + r, k = k0 + c;
                Bs[r][c] = (n < N && k < k_hi) ? B[(long long)k * sbk + (long long)n * sbn] : zero;
            }
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < MLP_BK; kk += 16) {
            uint32_t af[2][4], bf[4][2];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int r = wm + i * 16 + g;
                af[i][0] = *reinterpret_cast<const uint32_t *>(&As[r][kk + 2 * t4]);
                af[i][1] = *reinterpret_cast<const uint32_t *>(&As[r + 8][kk + 2 * t4]);
                af[i][2] = *reinterpret_cast<const uint32_t *>(&As[r][kk + 8 + 2 * t4]);
                af[i][3] = *reinterpret_cast<const uint32_t *>(&As[r + 8][kk + 8 + 2 * t4]);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int c = wn + j * 8 + g;
                bf[j][0] = *reinterpret_cast<const uint32_t *>(&Bs[c][kk + 2 * t4]);
                bf[j][1] = *reinterpret_cast<const uint32_t *>(&Bs[c][kk + 8 + 2 * t4]);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) mk_mma_bf16(acc[i][j], af[i], bf[j]);
        }
        __syncthreads();
    }
    // Epilogue. Accumulator r of a 16x8 tile: row g + 8*(r>>1), col 2*t4 + (r&1).
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int m = m0 + wm + i * 16 + g + 8 * (r >> 1);
                const int n = n0 + wn + j * 8 + 2 * t4 + (r & 1);
                if (m >= M || n >= N) continue;
                float v = acc[i][j][r];
                if (gridDim.z > 1) {
                    atomicAdd(&C[(long long)m * ldc + n], v);
                    continue;
                }
                if (flags & MK_GEMM_BIAS) v += bias[n];
                if (flags & MK_GEMM_ACCUMULATE) v += C[(long long)m * ldc + n];
                if (flags & MK_GEMM_RELU) v = fmaxf(v, 0.f);
                if (C) C[(long long)m * ldc + n] = v;
                if (Cb) Cb[(long long)m * ldcb + n] = __float2bfloat16(v);
            }
}

extern "C" int mk_gemm_bf16(int M, int N, int K, const void *A, long long sam, long long sak,
                            const void *B, long long sbk, long long sbn, float *C, long long ldc,
                            const float *bias, int flags, void *Cb, long long ldcb, void *stream)
{
    MK_REQUIRE(M > 0 && N > 0 && K > 0 && A && B, "mk_gemm_bf16: bad shape or null operand");
    MK_REQUIRE(C || Cb, "mk_gemm_bf16: no output");
    MK_REQUIRE(!(flags & MK_GEMM_ACCUMULATE) || C, "mk_gemm_bf16: accumulate needs C");
    MK_REQUIRE(!(flags & MK_GEMM_BIAS) || bias, "mk_gemm_bf16: bias flag without bias");
    dim3 grid((N + MLP_BN - 1) / MLP_BN, (M + MLP_BM - 1) / MLP_BM);
    MK_REQUIRE(grid.y < 65536, "mk_gemm_bf16: M too large");
    cudaStream_t st = mk_stream(stream);
    // Few output tiles and a long K (the weight gradients: K = batch): split
    // K over up to 8 slices that add into C, when the epilogue is a plain
    // store or accumulate into C.
    const int tiles = (int)(grid.x * grid.y);
    if (tiles < 64 && K >= 4 * MLP_BK && C && !Cb && !(flags & (MK_GEMM_BIAS | MK_GEMM_RELU))) {
        int z = std::min(8, std::min(K / (2 * MLP_BK), (128 + tiles - 1) / tiles));
        if (z > 1) {
            grid.z = (unsigned)z;
            if (!(flags & MK_GEMM_ACCUMULATE))
                MK_CHECK_CUDA(cudaMemset2DAsync(C, sizeof(float) * (size_t)ldc, 0,
                                                sizeof(float) * (size_t)N, (size_t)M, st));
        }
    }
    mk_gemm_bf16_kernel<<<grid, 128, 0, st>>>(
        M, N, K, static_cast<const __nv_bfloat16 *>(A), sam, sak,
        static_cast<const __nv_bfloat16 *>(B), sbk, sbn, C, ldc, bias, flags,
        static_cast<__nv_bfloat16 *>(Cb), ldcb);
    MK_CHECK_CUDA(cudaGetLastError());
    return MK_OK;
}

// features[b] = [x, y, sin(2 pi f_j x), cos(2 pi f_j x), sin(2 pi f_j y), cos(2 pi f_j y)]_j,
// f_j = f0 ratio^j (j = 0 .. nf-1), zero-padded to `width` columns, bf16.
__global__ void mk_fourier_kernel(int n, const float *__restrict__ xy, int nf, float f0,
                                  float ratio, int width, __nv_bfloat16 *__restrict__ out)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    const float x = xy[2 * b], y = xy[2 * b + 1];
    __nv_bfloat16 *o = out + (size_t)b * width;
    o[0] = __float2bfloat16(x);
    o[1] = __float2bfloat16(y);
    float f = f0;
    for (int j = 0; j < nf; ++j, f *= ratio) {
        float sx, cx, sy, cy;
        sincospif(2.f * f * x, &sx, &cx);
        sincospif(2.f * f * y, &sy, &cy);
        o[2 + 4 * j] = __float2bfloat16(sx);
        o[3 + 4 * j] = __float2bfloat16(cx);
        o[4 + 4 * j] = __float2bfloat16(sy);
        o[5 + 4 * j] = __float2bfloat16(cy);
    }
    for (int c = 2 + 4 * nf; c < width; ++c) o[c] = __float2bfloat16(0.f);
}

extern "C" int mk_fourier_features(int n, const float *xy, int n_freq, float f0, float ratio,
                                   int width, void *out, void *stream)
{
    MK_REQUIRE(n > 0 && xy && out && n_freq >= 0 && width >= 2 + 4 * n_freq && f0 > 0.f &&
                   ratio >= 1.f,
               "mk_fourier_features: bad arguments");
    mk_fourier_kernel<<<(n + 127) / 128, 128, 0, mk_stream(stream)>>>(
        n, xy, n_freq, f0, ratio, width, static_cast<__nv_bfloat16 *>(out));
    MK_CHECK_CUDA(cudaGetLastError());
    return MK_OK;
}

// g[i] = grad[i] * (pre[i] > 0), written as bf16 (the operand of the next
// backward GEMMs) and as float.
__global__ void mk_relu_bwd_kernel(long long n, const float *__restrict__ grad,
                                   const float *__restrict__ pre, float *__restrict__ gout,
                                   __nv_bfloat16 *__restrict__ gb)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float v = pre[i] > 0.f ? grad[i] : 0.f;
    if (gout) gout[i] = v;
    if (gb) gb[i] = __float2bfloat16(v);
}

extern "C" int mk_relu_backward(long long n, const float *grad, const float *pre, float *gout,
                                void *gout_bf16, void *stream)
{
    MK_REQUIRE(n > 0 && grad && pre && (gout || gout_bf16), "mk_relu_backward: bad arguments");
    mk_relu_bwd_kernel<<<(unsigned)((n + 255) / 256), 256, 0, mk_stream(stream)>>>(
        n, grad, pre, gout, static_cast<__nv_bfloat16 *>(gout_bf16));
    MK_CHECK_CUDA(cudaGetLastError());
    return MK_OK;
}

// db[n] = sum_m g[m, n]: block (x, y) sums 32 columns over the y-th slice
// of rows (8 warps, warp w taking rows w, w + 8, ..., four in flight), adds
// its 8 warp sums and then adds the result into db (zeroed first) with an
// atomic add: many blocks keep enough loads in flight for a tall, narrow g.
#define MK_COLSUM_ROWS 128
__global__ void __launch_bounds__(256) mk_colsum_kernel(int M, int N, const float *__restrict__ g,
                                                        long long g_stride, float *__restrict__ db,
                                                        long long db_stride)
{
    __shared__ float part[8][33];
    g += blockIdx.z * g_stride;             // group blockIdx.z
    db += blockIdx.z * db_stride;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int n = blockIdx.x * 32 + lane;
    const int m_lo = blockIdx.y * MK_COLSUM_ROWS, m_hi = min(M, m_lo + MK_COLSUM_ROWS);
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    if (n < N) {
        int m = m_lo + warp;
        for (; m + 24 < m_hi; m += 32) {
            s0 += g[(long long)m * N + n];
            s1 += g[(long long)(m + 8) * N + n];
            s2 += g[(long long)(m + 16) * N + n];
            s3 += g[(long long)(m + 24) * N + n];
        }
        for (; m < m_hi; m += 8) s0 += g[(long long)m * N + n];
    }
    part[warp][lane] = (s0 + s1) + (s2 + s3);
    __syncthreads();
    if (warp == 0 && n < N) {
        float s = 0.f;
#pragma unroll
        for (int w = 0; w < 8; ++w) s += part[w][lane];
        atomicAdd(&db[n], s);
    }
}

extern "C" int mk_bias_grad_groups(int groups, int M, int N, const float *g, long long g_stride,
                                   float *db, long long db_stride, void *stream)
{
    MK_REQUIRE(groups >= 1 && M > 0 && N > 0 && g && db, "mk_bias_grad: bad arguments");
    MK_REQUIRE(groups == 1 || db_stride >= N, "mk_bias_grad: groups' gradients overlap");
    dim3 grid((N + 31) / 32, (M + MK_COLSUM_ROWS - 1) / MK_COLSUM_ROWS, groups);
    MK_REQUIRE(grid.y < 65536 && groups < 65536, "mk_bias_grad: M or groups too large");
    cudaStream_t st = mk_stream(stream);
    for (int q = 0; q < groups; ++q)
        MK_CHECK_CUDA(cudaMemsetAsync(db + q * db_stride, 0, sizeof(float) * (size_t)N, st));
    mk_colsum_kernel<<<grid, 256, 0, st>>>(M, N, g, g_stride, db, db_stride);
    MK_CHECK_CUDA(cudaGetLastError());
    return MK_OK;
}

extern "C" int mk_bias_grad(int M, int N, const float *g, float *db, void *stream)
{
    return mk_bias_grad_groups(1, M, N, g, 0, db, 0, stream);
}

// Mean squared error over the n entries, each weighted by its column's
// weight when col_w is given (row-major, n_col columns):
// grad = 2 w (y - t) / n (float and bf16), per-block partial sums of
// w (y - t)^2 into part[blockIdx.x].
__global__ void mk_mse_kernel(long long n, int n_col, const float *__restrict__ y,
                              const float *__restrict__ t, const float *__restrict__ col_w,
                              float *__restrict__ grad, __nv_bfloat16 *__restrict__ gb,
                              double *__restrict__ part)
{
    __shared__ double red[256];
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double sq = 0.0;
    if (i < n) {
        const float d = y[i] - t[i];
        const float w = col_w ? col_w[i % n_col] : 1.f;
        const float gv = 2.f * w * d / (float)n;
        if (grad) grad[i] = gv;
        if (gb) gb[i] = __float2bfloat16(gv);
        sq = (double)w * d * d;
    }
    red[threadIdx.x] = sq;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

extern "C" int mk_mse(long long n, const float *y, const float *t, float *grad, void *grad_bf16,
                      double *partials, void *stream)
{
    MK_REQUIRE(n > 0 && y && t && partials, "mk_mse: bad arguments");
    mk_mse_kernel<<<(unsigned)((n + 255) / 256), 256, 0, mk_stream(stream)>>>(
        n, 1, y, t, nullptr, grad, static_cast<__nv_bfloat16 *>(grad_bf16), partials);
    MK_CHECK_CUDA(cudaGetLastError());
    return MK_OK;
}

extern "C" int mk_mse_weighted(long long n, int n_col, const float *y, const float *t,
                               const float *col_w, float *grad, void *grad_bf16,
                               double *partials, void *stream)
{
    MK_REQUIRE(n > 0 && n_col > 0 && n % n_col == 0 && y && t && col_w && partials,
               "mk_mse_weighted: bad arguments");
    mk_mse_kernel<<<(unsigned)((n + 255) / 256), 256, 0, mk_stream(stream)>>>(
        n, n_col, y, t, col_w, grad, static_cast<__nv_bfloat16 *>(grad_bf16), partials);
    MK_CHECK_CUDA(cudaGetLastError());
    return MK_OK;
}

// Adam on FP32 master weights; the bf16 copy the GEMMs read is refreshed.
__global__ void mk_adam_kernel(long long n, float *__restrict__ w, const float *__restrict__ g,
                               float *__restrict__ m, float *__restrict__ v,
                               __nv_bfloat16 *__restrict__ wb, float lr, float b1, float b2,
                               float eps, float c1, float c2, float wd)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i] + wd * w[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16(wi);
}

// The same step with its step number in device memory (t = *step + 1) and
// the learning rate from a schedule (lr_sched[*step - step0]), so that one
// captured training step replays with advancing steps.
__global__ void mk_adam_sched_kernel(long long n, float *__restrict__ w, const float *__restrict__ g,
                                     float *__restrict__ m, float *__restrict__ v,
                                     __nv_bfloat16 *__restrict__ wb,
                                     const float *__restrict__ lr_sched,
                                     const int *__restrict__ step, int step0, float b1, float b2,
                                     float eps, float wd)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int s = *step;
    const float t = (float)(s + 1);
    const float c1 = 1.f - powf(b1, t), c2 = 1.f - powf(b2, t);
    const float lr = lr_sched[s - step0];
    const float gi = g[i] + wd * w[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16(wi);
}

extern "C" int mk_adam_sched(long long n, float *w, const float *g, float *m, float *v,
                             void *w_bf16, const float *lr_sched, const int *step, int step0,
                             float beta1, float beta2, float eps, float weight_decay, void *stream)
{
    MK_REQUIRE(n > 0 && w && g && m && v && lr_sched && step && step0 >= 0,
               "mk_adam_sched: bad arguments");
    mk_adam_sched_kernel<<<(unsigned)((n + 255) / 256), 256, 0, mk_stream(stream)>>>(
        n, w, g, m, v, static_cast<__nv_bfloat16 *>(w_bf16), lr_sched, step, step0, beta1, beta2,
        eps, weight_decay);
    MK_CHECK_CUDA(cudaGetLastError());
    return MK_OK;
}

__global__ void mk_counter_add_kernel(int *c, int d) { *c += d; }

extern "C" int mk_counter_add(int *counter, int delta, void *stream)
{
    MK_REQUIRE(counter, "mk_counter_add: null counter");
    mk_counter_add_kernel<<<1, 1, 0, mk_stream(stream)>>>(counter, delta);
    MK_CHECK_CUDA(cudaGetLastError());
    return MK_OK;
}

extern "C" int mk_adam(long long n, float *w, const float *g, float *m, float *v, void *w_bf16,
                       float lr, float beta1, float beta2, float eps, int step, float weight_decay,
                       void *stream)
{
    MK_REQUIRE(n > 0 && w && g && m && v && step >= 1, "mk_adam: bad arguments");
    const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
    mk_adam_kernel<<<(unsigned)((n + 255) / 256), 256, 0, mk_stream(stream)>>>(
        n, w, g, m, v, static_cast<__nv_bfloat16 *>(w_bf16), lr, beta1, beta2, eps, c1, c2,
        weight_decay);
    MK_CHECK_CUDA(cudaGetLastError());
    return MK_OK;
}
