// Pipe-throughput microbenchmark: results per clock per SM of the MUFU sine,
// sin+cos, FRND, FFMA and packed FFMA2 (counted in FMAs). It measures the denominator of the split kernel's
// roofline on the GPU at hand. One wave of blocks, eight independent
// dependency chains per thread, per-block cycle counts from clock64(); every
// loop is bounded and every store in bounds (out holds grid*threads floats).
#include "mk_common.cuh"

#define PROBE_CHAINS 8
#define PROBE_THREADS 256
#define PROBE_BLOCKS_PER_SM 8

template <int KIND>
__global__ void __launch_bounds__(PROBE_THREADS) mk_probe_kernel(float *__restrict__ out, int iters,
                                                                 long long *__restrict__ cyc)
{
    float x[PROBE_CHAINS];
#pragma unroll
    for (int c = 0; c < PROBE_CHAINS; ++c) x[c] = 0.001f * (float)(threadIdx.x + 37 * c) + 0.1f;
    __syncthreads();
    const long long t0 = clock64();
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < PROBE_CHAINS; ++c) {
            if (KIND == 0) x[c] = __sinf(x[c]);
            if (KIND == 1) {
                float s, co;
                __sincosf(x[c], &s, &co);
                x[c] = s + co;
            }
            if (KIND == 2) x[c] = rintf(x[c] * 1.0001f) + 0.5f;
            if (KIND == 3) x[c] = fmaf(x[c], 0.9999f, 0.0001f);
            if (KIND == 4) {
                // packed FFMA2: two FP32 FMAs in one instruction, lanes
                // (x[c], x[c] + 1) so that neither half is dead
                unsigned long long v, m, a;
                asm("mov.b64 %0, {%1, %2};" : "=l"(v) : "f"(x[c]), "f"(x[c] + 1.f));
                asm("mov.b64 %0, {%1, %2};" : "=l"(m) : "f"(0.9999f), "f"(0.9998f));
                asm("mov.b64 %0, {%1, %2};" : "=l"(a) : "f"(0.0001f), "f"(0.0002f));
#pragma unroll
                for (int r = 0; r < 8; ++r)
                    asm volatile("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(v) : "l"(m), "l"(a));
                float lo, hi;
                asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
                x[c] = lo + hi;
            }
        }
    }
    const long long t1 = clock64();
    __syncthreads();
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < PROBE_CHAINS; ++c) s += x[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
    if (threadIdx.x == 0) cyc[blockIdx.x] = t1 - t0;
}

size_t mk_probe_scratch_bytes(int sms)
{
    const size_t blocks = (size_t)sms * PROBE_BLOCKS_PER_SM;
    return blocks * PROBE_THREADS * sizeof(float) + blocks * sizeof(long long) + 256;
}

extern "C" size_t mk_probe_workspace_size(void)
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return 0;
    return mk_probe_scratch_bytes(sms);
}

extern "C" int mk_probe_throughput(int kind, int iters, void *workspace, size_t ws_bytes,
                                   double *ops_per_clk_per_sm, void *stream)
{
    MK_REQUIRE(kind >= 0 && kind <= 4,
               "mk_probe_throughput: kind 0 sin, 1 sincos, 2 frnd, 3 ffma, 4 packed ffma2");
    MK_REQUIRE(iters >= 1 && iters <= (1 << 16), "mk_probe_throughput: iters in [1, 65536]");
    MK_REQUIRE(ops_per_clk_per_sm && workspace, "mk_probe_throughput: null argument");
    int dev = 0, sms = 0;
    MK_CHECK_CUDA(cudaGetDevice(&dev));
    MK_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const size_t need = mk_probe_scratch_bytes(sms);
    if (ws_bytes < need) {
        mk_set_error("mk_probe_throughput: workspace %zu bytes, need %zu", ws_bytes, need);
        return MK_ENOMEM;
    }
    const int grid = sms * PROBE_BLOCKS_PER_SM;
    float *out = static_cast<float *>(workspace);
    long long *cyc = reinterpret_cast<long long *>(static_cast<char *>(workspace) +
                                                   (size_t)grid * PROBE_THREADS * sizeof(float));
    cudaStream_t st = mk_stream(stream);
    for (int pass = 0; pass < 2; ++pass) {         // pass 0 warms clocks and caches
        const int it = pass == 0 ? 16 : iters;
        switch (kind) {
        case 0: mk_probe_kernel<0><<<grid, PROBE_THREADS, 0, st>>>(out, it, cyc); break;
        case 1: mk_probe_kernel<1><<<grid, PROBE_THREADS, 0, st>>>(out, it, cyc); break;
        case 2: mk_probe_kernel<2><<<grid, PROBE_THREADS, 0, st>>>(out, it, cyc); break;
        case 3: mk_probe_kernel<3><<<grid, PROBE_THREADS, 0, st>>>(out, it, cyc); break;
        default: mk_probe_kernel<4><<<grid, PROBE_THREADS, 0, st>>>(out, it, cyc); break;
        }
        MK_CHECK_CUDA(cudaGetLastError());
    }
    long long *h = new long long[grid];
    const cudaError_t e = cudaMemcpyAsync(h, cyc, sizeof(long long) * grid, cudaMemcpyDeviceToHost, st);
    const cudaError_t e2 = e == cudaSuccess ? cudaStreamSynchronize(st) : e;
    if (e2 != cudaSuccess) {
        delete[] h;
        mk_set_error("mk_probe_throughput: %s", cudaGetErrorString(e2));
        return MK_ECUDA;
    }
    long long mx = 1;
    for (int i = 0; i < grid; ++i) mx = h[i] > mx ? h[i] : mx;
    delete[] h;
    // sincos: two MUFU results; ffma2: 8 packed instructions of 2 FMAs each,
    // counted as FMAs (plus the lane moves and the final add, not counted)
    const double per_call = kind == 1 ? 2.0 : (kind == 4 ? 16.0 : 1.0);
    const double ops = (double)grid * PROBE_THREADS * iters * PROBE_CHAINS * per_call;
    *ops_per_clk_per_sm = ops / ((double)mx * sms);
    return MK_OK;
}
