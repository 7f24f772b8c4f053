// FP32 split-phase kinematic sum over Morton-ordered atom tiles (sm_103a).
//
// The phase of atom a = o + d (o its tile origin) at pixel P splits as
//   k (b.a + |P - a|) = k |P|                                 per pixel, FP64 phasor
//                     + k (b.o + |P - o| - |P|)                per (tile, pixel), FP64
//                     + k (b.d + |P - o - d| - |P - o|)        per term, FP32
// with |P - o| - |P| = -u.o + (|o|^2 - (u.o)^2) / 2|P| + O(|o|^3/|P|^2) and
// |P - o - d| - |P - o| = -u'.d + (|d|^2 - (u'.d)^2) / 2|P - o| + O(|d|^3/|P|^2),
// u = P/|P|, u' = (P - o)/|P - o| = u - (o - (u.o) u)/|P| + O(|o|^2/|P|^2).
// Everything is carried in cycles (phase / 2 pi). The dominant part of the
// (tile, pixel) phase, (k/2pi)(b - u).o, is an FP64 dot product of the
// per-pixel vector qc (from mk_pixels_prepare) with the FP64 tile origin,
// reduced mod 1 in FP64; the rest is small and FP32. Inside the tile the
// term phase is w.D (+ the |d|^2 term when `FRESNEL`), w = b - u', D the
// float32 offset in cycles: 3 FMA, a mod-1 reduction, and sin/cos on the MUFU.
//
// The direction-dependent factor (f0 + f' + i f'') exp(-B s^2) sqrt(P_pol)
// [R0/r] is evaluated once per (tile, pixel) at the tile direction u'; its
// change across a tile is ~|d|/|P| relative. Per-tile sums are folded into
// the per-pixel accumulators with Kahan compensation; slices of the tile
// range write partial fields that an FP64 pass adds in a fixed order, so the
// result does not depend on scheduling.
#include <algorithm>

#include "mk_common.cuh"

static __device__ int g_split_status;

static int mk_split_read_status(cudaStream_t st)
{
    int v = 0, zero = 0;
    if (cudaMemcpyFromSymbolAsync(&v, g_split_status, sizeof(int), 0, cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaMemcpyToSymbolAsync(g_split_status, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        mk_set_error("mk_sync_status: cannot read the split kernel status word");
        return MK_ECUDA;
    }
    if (v == MK_DEV_TIMEOUT_TMA) {
        mk_set_error("split-phase kernel: a tile copy did not complete within its time limit");
        return MK_ETIMEOUT;
    }
    return MK_OK;
}

struct MkSplitArgs {
    MkSpecies sp;
    int n_pix, n_tiles, tiles_per_slice, tile_atoms;
    const double *qc;
    const double *qcut;
    const float *uf;
    const double4 *origin;
    const int *tspecies;
    const float4 *tpos;
    const float2 *tamp;
    double2 *partial;
    int *status;
    float bx, by, bz;
    float kappa;       // k / 2 pi [cycles/m]
    float k;           // [1/m]
    float s2fac;       // (k 0.25e-10 / pi)^2: s^2 = s2fac |b - u'|^2 [1/A^2]
    int apply_pol, decay, remove_forward;
    float pdeg, ex, ey, ez;
};

#define TWO_PI_F 6.28318530717958647692f

// Scattering factor of species s at direction u' = (upx, upy, upz); w = b - u'.
__device__ __forceinline__ float2 mk_factor(const MkSplitArgs &A, int s, float wx, float wy,
                                           float wz, float upx, float upy, float upz, float qcut,
                                           float decay_ratio)
{
    const float w2 = fmaf(wz, wz, fmaf(wy, wy, wx * wx));
    const float s2 = A.s2fac * w2;
    const float *wk = A.sp.wk[s];
    float f0 = wk[5];
#pragma unroll
    for (int i = 0; i < 5; ++i) f0 = fmaf(wk[i], __expf(-wk[6 + i] * s2), f0);
    float fr = f0 + A.sp.anr[s], fi = A.sp.ani[s];
    if (A.remove_forward && A.k * sqrtf(w2) < qcut) {
        fr -= A.sp.f0z[s] + A.sp.anr[s];
        fi -= A.sp.ani[s];
    }
    float scale = 1.f;
    if (A.sp.has_dw) scale = __expf(-A.sp.dwb[s] * s2);
    if (A.apply_pol) {
        const float dotv = fmaf(A.bz, upz, fmaf(A.by, upy, A.bx * upx));
        const float er = fmaf(A.ez, upz, fmaf(A.ey, upy, A.ex * upx));
        float P = 0.5f * (1.f - A.pdeg) * fmaf(dotv, dotv, 1.f) + A.pdeg * fmaf(-er, er, 1.f);
        P = fminf(1.f, fmaxf(0.f, P));
        scale *= sqrtf(P);
    }
    if (A.decay) scale *= decay_ratio;
    return make_float2(fr * scale, fi * scale);
}

template <int NT, int PIX, bool FRESNEL, bool CPLX>
__global__ void __launch_bounds__(NT) mk_split_kernel(const __grid_constant__ MkSplitArgs A)
{
    extern __shared__ __align__(128) unsigned char smem[];
    const int T = A.tile_atoms;
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    float4 *s_pos = reinterpret_cast<float4 *>(smem + 128);     // [2][T]
    float2 *s_amp = reinterpret_cast<float2 *>(s_pos + 2 * T);   // [2][T]
    const int tid = threadIdx.x;
    const int n = A.n_pix;
    const int t_lo = blockIdx.y * A.tiles_per_slice;
    const int t_hi = min(A.n_tiles, t_lo + A.tiles_per_slice);
    const uint32_t tile_bytes = (uint32_t)T * (uint32_t)(sizeof(float4) + sizeof(float2));

    if (tid == 0) {
        mk_mbar_init(&bar[0], 1);
        mk_mbar_init(&bar[1], 1);
        mk_fence_barrier_init();
    }
    __syncthreads();
    if (tid == 0) {
        for (int b = 0; b < 2 && t_lo + b < t_hi; ++b) {
            mk_mbar_expect_tx(&bar[b], tile_bytes);
            mk_tma_load_1d(s_pos + b * T, A.tpos + (size_t)(t_lo + b) * T, T * sizeof(float4), &bar[b]);
            mk_tma_load_1d(s_amp + b * T, A.tamp + (size_t)(t_lo + b) * T, T * sizeof(float2), &bar[b]);
        }
    }

    int pix[PIX];
    float accr[PIX], acci[PIX], cmpr[PIX], cmpi[PIX];
#pragma unroll
    for (int p = 0; p < PIX; ++p) {
        pix[p] = blockIdx.x * (NT * PIX) + p * NT + tid;
        accr[p] = acci[p] = cmpr[p] = cmpi[p] = 0.f;
    }

    for (int t = t_lo, it = 0; t < t_hi; ++t, ++it) {
        const int buf = it & 1;
        const uint32_t parity = (uint32_t)(it >> 1) & 1u;
        const double4 o = A.origin[t];
        const float ox = (float)o.x, oy = (float)o.y, oz = (float)o.z;
        // Per (tile, pixel): w = b - u' in registers for the atom loop.
        float wx[PIX], wy[PIX], wz[PIX], hq[PIX];
#pragma unroll
        for (int p = 0; p < PIX; ++p) {
            const int q = min(pix[p], n - 1);
            const float ux = A.uf[q], uy = A.uf[n + q], uz = A.uf[2 * n + q], iR = A.uf[3 * n + q];
            const float uo = fmaf(uz, oz, fmaf(uy, oy, ux * ox));
            const float upx = ux - (ox - uo * ux) * iR;
            const float upy = uy - (oy - uo * uy) * iR;
            const float upz = uz - (oz - uo * uz) * iR;
            wx[p] = A.bx - upx;
            wy[p] = A.by - upy;
            wz[p] = A.bz - upz;
            // 1 / (2 kappa |P - o|) for the |d|^2 term (D is in cycles).
            hq[p] = FRESNEL ? 0.5f * iR / (A.kappa * fmaf(-uo, iR, 1.f)) : 0.f;
        }
        const bool ok = mk_mbar_wait_bounded(&bar[buf], parity, MK_WAIT_LIMIT_NS);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                atomicExch(A.status, MK_DEV_TIMEOUT_TMA);
                // Let any copy still in flight land before the block's shared
                // memory is released (bounded as well).
                mk_mbar_wait_bounded(&bar[0], 0, MK_WAIT_LIMIT_NS / 2);
                mk_mbar_wait_bounded(&bar[1], 0, MK_WAIT_LIMIT_NS / 2);
            }
            return;
        }
        const float4 *P = s_pos + buf * T;
        const float2 *E = s_amp + buf * T;
        float csr[PIX], csi[PIX];
#pragma unroll
        for (int p = 0; p < PIX; ++p) csr[p] = csi[p] = 0.f;
#pragma unroll 4
        for (int j = 0; j < T; ++j) {
            const float4 a = P[j];
            const float2 e = E[j];
            float db = 0.f;
            if (FRESNEL) db = fmaf(a.z, A.bz, fmaf(a.y, A.by, a.x * A.bx));
#pragma unroll
            for (int p = 0; p < PIX; ++p) {
                float lin = fmaf(a.z, wz[p], fmaf(a.y, wy[p], a.x * wx[p]));
                if (FRESNEL) {
                    const float sp = db - lin;
                    lin = fmaf(fmaf(-sp, sp, a.w), hq[p], lin);
                }
                const float r = lin - rintf(lin);
                float sn, cs;
                __sincosf(r * TWO_PI_F, &sn, &cs);
                if (CPLX) {
                    csr[p] = fmaf(e.x, cs, fmaf(-e.y, sn, csr[p]));
                    csi[p] = fmaf(e.x, sn, fmaf(e.y, cs, csi[p]));
                } else {
                    csr[p] = fmaf(e.x, cs, csr[p]);
                    csi[p] = fmaf(e.x, sn, csi[p]);
                }
            }
        }
        __syncthreads();   // every thread is done with buffer `buf`
        if (tid == 0 && t + 2 < t_hi) {
            mk_fence_proxy_async();
            mk_mbar_expect_tx(&bar[buf], tile_bytes);
            mk_tma_load_1d(s_pos + buf * T, A.tpos + (size_t)(t + 2) * T, T * sizeof(float4), &bar[buf]);
            mk_tma_load_1d(s_amp + buf * T, A.tamp + (size_t)(t + 2) * T, T * sizeof(float2), &bar[buf]);
        }
        // Fold: tile sum x factor x exp(2 pi i phi0), Kahan-compensated.
        const int s = A.tspecies[t];
        const float oo = fmaf(oz, oz, fmaf(oy, oy, ox * ox));
#pragma unroll
        for (int p = 0; p < PIX; ++p) {
            const int q = min(pix[p], n - 1);
            const float ux = A.uf[q], uy = A.uf[n + q], uz = A.uf[2 * n + q], iR = A.uf[3 * n + q];
            const float uo = fmaf(uz, oz, fmaf(uy, oy, ux * ox));
            const double q0 = A.qc[q] * o.x + A.qc[n + q] * o.y + A.qc[2 * n + q] * o.z;
            float ph = (float)(q0 - rint(q0)) + A.kappa * 0.5f * fmaf(-uo, uo, oo) * iR;
            ph -= rintf(ph);
            float s0, c0;
            __sincosf(ph * TWO_PI_F, &s0, &c0);
            const float2 F = mk_factor(A, s, wx[p], wy[p], wz[p], A.bx - wx[p], A.by - wy[p],
                                       A.bz - wz[p], (float)A.qcut[q],
                                       1.f / fmaf(-uo, iR, 1.f));
            const float gr = F.x * c0 - F.y * s0, gi = F.x * s0 + F.y * c0;
            const float tr = csr[p] * gr - csi[p] * gi;
            const float ti = csr[p] * gi + csi[p] * gr;
            float y = tr - cmpr[p];
            float z = accr[p] + y;
            cmpr[p] = (z - accr[p]) - y;
            accr[p] = z;
            y = ti - cmpi[p];
            z = acci[p] + y;
            cmpi[p] = (z - acci[p]) - y;
            acci[p] = z;
        }
    }
#pragma unroll
    for (int p = 0; p < PIX; ++p) {
        if (pix[p] < n)
            A.partial[(size_t)blockIdx.y * n + pix[p]] =
                make_double2((double)accr[p] - (double)cmpr[p], (double)acci[p] - (double)cmpi[p]);
    }
}

// Test hook for the bounded-wait path: one block waits on an mbarrier that
// no copy and no thread ever completes, gives up after `limit_ns`, records
// the timeout in the status word and returns. Nothing is in flight, so the
// context stays usable.
__global__ void mk_wait_probe_kernel(uint64_t limit_ns, int *status)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mk_mbar_init(&bar, 1);
        mk_fence_barrier_init();
    }
    __syncthreads();
    const bool ok = mk_mbar_wait_bounded(&bar, 0, limit_ns);
    if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicExch(status, MK_DEV_TIMEOUT_TMA);
}

extern "C" int mk_debug_wait_timeout(uint64_t limit_ns, void *stream)
{
    MK_REQUIRE(limit_ns > 0 && limit_ns <= 1000000000ull,
               "mk_debug_wait_timeout: limit must be in (0, 1 s]");
    mk_register_status_reader(mk_split_read_status);
    int *status = nullptr;
    MK_CHECK_CUDA(cudaGetSymbolAddress((void **)&status, g_split_status));
    mk_wait_probe_kernel<<<1, 32, 0, mk_stream(stream)>>>(limit_ns, status);
    MK_CHECK_CUDA(cudaGetLastError());
    return MK_OK;
}

// out[p] (+)= scale * phasor[p] * sum_s partial[s][p], slices added in order in FP64.
__global__ void mk_reduce_kernel(const double2 *__restrict__ partial, int slices, int n_pix,
                                 const double2 *__restrict__ phasor, double scale,
                                 double2 *__restrict__ out, int accumulate)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_pix) return;
    double re = 0.0, im = 0.0;
    for (int s = 0; s < slices; ++s) {
        const double2 v = partial[(size_t)s * n_pix + p];
        re += v.x;
        im += v.y;
    }
    if (phasor) {
        const double2 e = phasor[p];
        const double r2 = re * e.x - im * e.y, i2 = re * e.y + im * e.x;
        re = r2;
        im = i2;
    }
    re *= scale;
    im *= scale;
    if (accumulate) {
        const double2 o = out[p];
        re += o.x;
        im += o.y;
    }
    out[p] = make_double2(re, im);
}

int mk_launch_reduce(const double2 *partial, int slices, int n_pix, const double2 *phasor,
                     double scale, double2 *out, int accumulate, cudaStream_t st)
{
    mk_reduce_kernel<<<(n_pix + 255) / 256, 256, 0, st>>>(partial, slices, n_pix, phasor, scale, out,
                                                          accumulate);
    MK_CHECK_CUDA(cudaGetLastError());
    return MK_OK;
}

// ----------------------------------------------------------------- launch
typedef void (*mk_split_fn)(const MkSplitArgs);

template <int NT, int PIX>
static mk_split_fn mk_pick3(bool fresnel, bool cplx)
{
    if (fresnel) return cplx ? mk_split_kernel<NT, PIX, true, true> : mk_split_kernel<NT, PIX, true, false>;
    return cplx ? mk_split_kernel<NT, PIX, false, true> : mk_split_kernel<NT, PIX, false, false>;
}

static mk_split_fn mk_pick(int nt, int pix, bool fresnel, bool cplx)
{
#define MK_PIX_CASES(NT_)                                                  \
    switch (pix) {                                                         \
    case 1: return mk_pick3<NT_, 1>(fresnel, cplx);                        \
    case 2: return mk_pick3<NT_, 2>(fresnel, cplx);                        \
    case 4: return mk_pick3<NT_, 4>(fresnel, cplx);                        \
    case 8: return mk_pick3<NT_, 8>(fresnel, cplx);                        \
    default: return nullptr;                                               \
    }
    switch (nt) {
    case 64: MK_PIX_CASES(64)
    case 128: MK_PIX_CASES(128)
    case 256: MK_PIX_CASES(256)
    default: return nullptr;
    }
#undef MK_PIX_CASES
}

static size_t mk_split_smem(int T) { return 128 + (size_t)2 * T * (sizeof(float4) + sizeof(float2)); }

// Slices so that the grid fills the GPU in whole waves: minimise
// waves(slices) x tiles-per-slice over the feasible range.
static int mk_auto_slices(int blocks_x, int n_tiles, int resident)
{
    int best = 1;
    double best_cost = 1e300;
    const int cap = std::max(1, std::min(n_tiles, 8192));
    for (int s = 1; s <= cap; ++s) {
        const int per = (n_tiles + s - 1) / s;
        const int s_eff = (n_tiles + per - 1) / per;
        if (s_eff != s) continue;
        const double blocks = (double)blocks_x * s;
        const double waves = std::ceil(blocks / resident);
        const double cost = waves * per + 0.02 * s;   // small bias against extra partials
        if (cost < best_cost) {
            best_cost = cost;
            best = s;
        }
    }
    return best;
}

extern "C" size_t mk_sum_workspace_size(int n_pix, int slices)
{
    if (n_pix <= 0 || slices <= 0) return 256;
    return sizeof(double2) * (size_t)n_pix * (size_t)slices;
}

static int mk_split_config(const mk_tiles *tiles, const mk_pixels *px, const mk_launch *launch,
                           int cplx, int fresnel, mk_split_fn *fn_out, int *slices_out,
                           int *per_out)
{
    const int n_pix = px->ny * px->nz;
    mk_split_fn fn = mk_pick(launch->threads, launch->pix_per_thread, fresnel != 0, cplx != 0);
    MK_REQUIRE(fn, "mk_kin_split_f32: unsupported launch shape threads=%d pix=%d", launch->threads,
               launch->pix_per_thread);
    const size_t smem = mk_split_smem(tiles->tile_atoms);
    MK_CHECK_CUDA(cudaFuncSetAttribute((const void *)fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
    const int blocks_x = (n_pix + launch->threads * launch->pix_per_thread - 1) /
                         (launch->threads * launch->pix_per_thread);
    int slices = launch->slices;
    if (slices <= 0) {
        int dev = 0, sms = 152, bps = 1;
        MK_CHECK_CUDA(cudaGetDevice(&dev));
        MK_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        MK_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, (const void *)fn,
                                                                    launch->threads, smem));
        MK_REQUIRE(bps >= 1, "mk_kin_split_f32: launch shape does not fit on an SM");
        slices = mk_auto_slices(blocks_x, tiles->n_tiles, sms * bps);
    }
    slices = std::max(1, std::min(slices, tiles->n_tiles));
    const int per = (tiles->n_tiles + slices - 1) / slices;
    *slices_out = (tiles->n_tiles + per - 1) / per;
    *per_out = per;
    *fn_out = fn;
    return MK_OK;
}

extern "C" int mk_split_plan(const mk_tiles *tiles, const mk_pixels *px, const mk_launch *launch,
                             int *slices_out)
{
    MK_REQUIRE(tiles && px && launch && slices_out, "mk_split_plan: null argument");
    MK_REQUIRE(px->ny > 0 && px->nz > 0, "mk_split_plan: bad detector shape");
    if (tiles->n_tiles <= 0) {
        *slices_out = 0;
        return MK_OK;
    }
    mk_split_fn fn;
    int per;
    const int fresnel = launch->fresnel < 0 ? 1 : launch->fresnel;
    return mk_split_config(tiles, px, launch, launch->amp_real ? 0 : 1, fresnel, &fn, slices_out, &per);
}

extern "C" int mk_kin_split_f32(const mk_tiles *tiles, const mk_species *spc,
                                const mk_physics *phys, const mk_pixels *px,
                                const mk_launch *launch, double *out, int accumulate,
                                void *workspace, size_t ws_bytes, void *stream)
{
    MK_REQUIRE(tiles && spc && phys && px && launch && out, "mk_kin_split_f32: null argument");
    const int64_t np64 = (int64_t)px->ny * px->nz;
    MK_REQUIRE(px->ny > 0 && px->nz > 0 && np64 < (1ll << 31), "mk_kin_split_f32: bad detector shape");
    MK_REQUIRE(px->qc && px->qcut && px->uf && px->phasor, "mk_kin_split_f32: pixels not prepared");
    MK_REQUIRE(phys->k > 0.0, "mk_kin_split_f32: k must be positive");
    const int T = tiles->tile_atoms;
    MK_REQUIRE(T >= 128 && T <= 4096 && (T & (T - 1)) == 0, "mk_kin_split_f32: bad tile_atoms %d", T);
    const int n_pix = (int)np64;
    cudaStream_t st = mk_stream(stream);
    if (tiles->n_tiles <= 0) {
        if (!accumulate) MK_CHECK_CUDA(cudaMemsetAsync(out, 0, sizeof(double2) * (size_t)n_pix, st));
        return MK_OK;
    }
    MK_REQUIRE(tiles->origin && tiles->species && tiles->pos && tiles->amp,
               "mk_kin_split_f32: null tile buffer");
    MK_REQUIRE(((uintptr_t)tiles->pos & 15) == 0 && ((uintptr_t)tiles->amp & 15) == 0,
               "mk_kin_split_f32: tile arrays must be 16-byte aligned");
    MkSplitArgs A;
    int rc = mk_species_pack(spc, &A.sp);
    if (rc != MK_OK) return rc;
    mk_register_status_reader(mk_split_read_status);
    const int fresnel = launch->fresnel < 0 ? 1 : launch->fresnel;
    const int cplx = launch->amp_real ? 0 : 1;
    mk_split_fn fn;
    int slices, per;
    rc = mk_split_config(tiles, px, launch, cplx, fresnel, &fn, &slices, &per);
    if (rc != MK_OK) return rc;
    const size_t need = mk_sum_workspace_size(n_pix, slices);
    if (!workspace || ws_bytes < need) {
        mk_set_error("mk_kin_split_f32: workspace %zu bytes, need %zu (slices=%d)", ws_bytes, need,
                     slices);
        return MK_ENOMEM;
    }
    int *status = nullptr;
    MK_CHECK_CUDA(cudaGetSymbolAddress((void **)&status, g_split_status));
    A.n_pix = n_pix;
    A.n_tiles = tiles->n_tiles;
    A.tiles_per_slice = per;
    A.tile_atoms = T;
    A.qc = px->qc;
    A.qcut = px->qcut;
    A.uf = px->uf;
    A.origin = reinterpret_cast<const double4 *>(tiles->origin);
    A.tspecies = tiles->species;
    A.tpos = reinterpret_cast<const float4 *>(tiles->pos);
    A.tamp = reinterpret_cast<const float2 *>(tiles->amp);
    A.partial = static_cast<double2 *>(workspace);
    A.status = status;
    A.bx = (float)phys->beam_dir[0];
    A.by = (float)phys->beam_dir[1];
    A.bz = (float)phys->beam_dir[2];
    A.kappa = (float)(phys->k / MK_TWO_PI);
    A.k = (float)phys->k;
    const double sf = phys->k * 0.25e-10 / MK_PI;
    A.s2fac = (float)(sf * sf);
    A.apply_pol = phys->apply_pol;
    A.decay = phys->spherical_decay;
    A.remove_forward = phys->remove_forward;
    A.pdeg = (float)phys->pol_deg;
    A.ex = (float)phys->pol_e[0];
    A.ey = (float)phys->pol_e[1];
    A.ez = (float)phys->pol_e[2];
    const int blocks_x = (n_pix + launch->threads * launch->pix_per_thread - 1) /
                         (launch->threads * launch->pix_per_thread);
    dim3 grid(blocks_x, slices);
    fn<<<grid, launch->threads, mk_split_smem(T), st>>>(A);
    MK_CHECK_CUDA(cudaGetLastError());
    return mk_launch_reduce(A.partial, slices, n_pix, reinterpret_cast<const double2 *>(px->phasor),
                            MK_R_E, reinterpret_cast<double2 *>(out), accumulate, st);
}
