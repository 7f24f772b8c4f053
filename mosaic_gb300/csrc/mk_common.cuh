// Shared device/host helpers of libmosaic_kin (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cmath>

#include "../../include/mosaic_kin.h"

// ---------------------------------------------------------------- errors
// Thread-local message behind mk_last_error(); every entry point returns a
// status code and never aborts.
void mk_set_error(const char *fmt, ...);

#define MK_CHECK_CUDA(call)                                                          \
    do {                                                                             \
        cudaError_t e_ = (call);                                                     \
        if (e_ != cudaSuccess) {                                                     \
            mk_set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
            return MK_ECUDA;                                                         \
        }                                                                            \
    } while (0)

#define MK_REQUIRE(cond, ...)                                                        \
    do {                                                                             \
        if (!(cond)) {                                                               \
            mk_set_error(__VA_ARGS__);                                               \
            return MK_EINVAL;                                                        \
        }                                                                            \
    } while (0)

static inline cudaStream_t mk_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// Device-side error codes written to a status word by kernels that wait on
// an mbarrier (the wait is bounded; on expiry the kernel records this and
// returns instead of trapping or spinning forever).
#define MK_DEV_TIMEOUT_TMA 1

// Registered by each translation unit that owns a status word; read and
// cleared by mk_sync_status().
typedef int (*mk_status_reader)(cudaStream_t);
void mk_register_status_reader(mk_status_reader fn);

// ------------------------------------------------------------- constants
#define MK_R_E 2.81794092e-15        /* classical electron radius [m] (Beam.py:704) */
#define MK_TWO_PI 6.283185307179586
#define MK_PI 3.14159265358979323846

// Analyser acceptance (Beam.py:2350-2378) from x = |r_hat - c|^2, the squared
// chord between the unit atom->pixel direction and the analyser axis; the
// angle is theta = 2 asin(sqrt(x) / 2), and x resolves small angles where
// cos(theta) cannot. kind 1 top-hat: 1 for x <= x_accept (theta <= alpha,
// x_accept = 4 sin^2(alpha / 2)), else 0; kind 2 Darwin:
// 1 / (1 + (theta / hw)^2), 1 when hw <= 0.
__host__ __device__ __forceinline__ double mk_analyser_factor(int kind, double x, double x_accept,
                                                            double hw)
{
    if (kind == 1) return x <= x_accept ? 1.0 : 0.0;
    if (kind == 2 && hw > 0.0) {
        const double h = 0.5 * sqrt(x > 0.0 ? x : 0.0);
        const double th = 2.0 * asin(h < 1.0 ? h : 1.0) / hw;
        return 1.0 / (1.0 + th * th);
    }
    return 1.0;
}

// Checks and unpacks the analyser fields of mk_physics.
static inline int mk_analyser_pack(const mk_physics *phys, int *kind, double *ax, double *ay,
                                   double *az, double *x_accept, double *hw)
{
    *kind = phys->analyser;
    *ax = *ay = *az = *x_accept = *hw = 0.0;
    if (!phys->analyser) return MK_OK;
    MK_REQUIRE(phys->analyser == 1 || phys->analyser == 2, "analyser kind must be 0, 1 or 2");
    const double *c = phys->analyser_dir;
    const double n = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    MK_REQUIRE(n > 0.0 && fabs(n - 1.0) < 1e-6, "analyser_dir must be a unit vector");
    MK_REQUIRE(phys->analyser_accept >= 0.0, "analyser acceptance must be >= 0");
    *ax = c[0] / n; *ay = c[1] / n; *az = c[2] / n;
    const double h = sin(0.5 * (phys->analyser_accept < MK_PI ? phys->analyser_accept : MK_PI));
    *x_accept = 4.0 * h * h;
    *hw = phys->analyser_halfwidth;
    return MK_OK;
}

// Per-species table passed by value to kernels.
struct MkSpecies {
    int n;
    int has_dw;
    float wk[MK_MAX_SPECIES][11];
    float f0z[MK_MAX_SPECIES];
    float anr[MK_MAX_SPECIES];
    float ani[MK_MAX_SPECIES];
    float dwb[MK_MAX_SPECIES];
};

static inline int mk_species_pack(const mk_species *sp, MkSpecies *out)
{
    if (!sp || sp->n_species < 1 || sp->n_species > MK_MAX_SPECIES || !sp->wk || !sp->f0_zero ||
        !sp->anom_re || !sp->anom_im) {
        mk_set_error("species table: need 1..%d species with wk, f0_zero, anom_re, anom_im",
                     MK_MAX_SPECIES);
        return MK_EINVAL;
    }
    out->n = sp->n_species;
    out->has_dw = sp->dw_b != nullptr;
    for (int s = 0; s < MK_MAX_SPECIES; ++s) {
        for (int i = 0; i < 11; ++i) out->wk[s][i] = s < sp->n_species ? sp->wk[11 * s + i] : 0.f;
        out->f0z[s] = s < sp->n_species ? sp->f0_zero[s] : 0.f;
        out->anr[s] = s < sp->n_species ? sp->anom_re[s] : 0.f;
        out->ani[s] = s < sp->n_species ? sp->anom_im[s] : 0.f;
        out->dwb[s] = (s < sp->n_species && sp->dw_b) ? sp->dw_b[s] : 0.f;
    }
    return MK_OK;
}

// --------------------------------------------------- TMA / mbarrier (PTX)
__device__ __forceinline__ uint32_t mk_smem_addr(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mk_mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mk_smem_addr(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void mk_fence_barrier_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mk_fence_proxy_async()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mk_mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mk_smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}

// 1-D bulk copy global -> shared, completion counted on `bar` (bytes).
// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void mk_tma_load_1d(void *dst, const void *src, uint32_t bytes,
                                               uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            mk_smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(mk_smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool mk_mbar_test(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(mk_smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t mk_globaltimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Wait for phase `parity` of `bar` for at most `limit_ns`; false on expiry.
__device__ __forceinline__ bool mk_mbar_wait_bounded(uint64_t *bar, uint32_t parity,
                                                     uint64_t limit_ns)
{
    if (mk_mbar_test(bar, parity)) return true;
    const uint64_t t0 = mk_globaltimer();
    for (;;) {
        if (mk_mbar_test(bar, parity)) return true;
        if (mk_globaltimer() - t0 > limit_ns) return false;
        __nanosleep(32);
    }
}

#define MK_WAIT_LIMIT_NS 2000000000ull /* 2 s: a tile copy takes microseconds */
