// Free-space angular-spectrum propagation of the detector field: padding,
// the transfer-function multiply on the spectrum, and the centre crop fused
// with |A|^2. The FFTs in between are cuFFT (through the caller).
//
// Transfer function (the reference's prop_mul_kernel, MOSAIC Beam.py:4747-4834):
//   kt = (ky + kgy, kz + kgz), kt^2 <= k^2:
//     H = exp(i [ -z kt^2 / (sqrt(k^2 - kt^2) + k) + z (k - kga) ])
//   otherwise (evanescent):
//     H = exp(-|z| sqrt(kt^2 - k^2)) exp(-i z kga)
// with ky, kz the FFT frequencies 2 pi fftfreq(N, d). The phase is formed
// and reduced in FP64 (the evanescent carrier z kga is ~1e10 rad), then
// sin/cos in FP64: the multiply is one pass over the spectrum, so its cost
// is memory traffic, not arithmetic.
#include <algorithm>

#include "mk_common.cuh"

__device__ __forceinline__ double mk_fftfreq(int i, int n, double d)
{
    const int half = (n - 1) / 2 + 1;      // numpy.fft.fftfreq ordering
    const int m = i < half ? i : i - n;
    return (double)m / ((double)n * d);
}

// Pad (nz, ny) into (nz2, ny2) centred at (z0, y0): edge replication
// (mode 0) or a constant (mode 1).
__global__ void mk_prop_pad_kernel(const float2 *__restrict__ in, int ny, int nz,
                                   float2 *__restrict__ out, int ny2, int nz2, int y0, int z0,
                                   int mode, float2 cval)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= ny2 || y >= nz2) return;
    const int sx = x - y0, sz = y - z0;
    float2 v;
    if (mode == 1 && (sx < 0 || sx >= ny || sz < 0 || sz >= nz)) {
        v = cval;
    } else {
        v = in[min(max(sz, 0), nz - 1) * ny + min(max(sx, 0), ny - 1)];
    }
    out[(size_t)y * ny2 + x] = v;
}

__global__ void mk_prop_mul_kernel(float2 *__restrict__ F, int ny2, int nz2, double dy, double dz,
                                   double k, double z, double kga, double kgy, double kgz)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= ny2 || y >= nz2) return;
    const double a = MK_TWO_PI * mk_fftfreq(x, ny2, dy) + kgy;
    const double b = MK_TWO_PI * mk_fftfreq(y, nz2, dz) + kgz;
    const double kt2 = a * a + b * b, kx2 = k * k - kt2;
    double ph, amp;
    if (kx2 >= 0.0) {
        ph = -z * kt2 / (sqrt(kx2) + k) + z * (k - kga);
        amp = 1.0;
    } else {
        amp = exp(-fabs(z) * sqrt(-kx2));
        ph = fmod(-z * kga, MK_TWO_PI);
    }
    double s, c;
    sincos(ph, &s, &c);
    const size_t i = (size_t)y * ny2 + x;
    const float2 g = F[i];
    const double hr = amp * c, hi = amp * s;
    F[i] = make_float2((float)(g.x * hr - g.y * hi), (float)(g.x * hi + g.y * hr));
}

// Centre crop of the inverse transform, fused with |A|^2; `scale` applies
// the inverse FFT's normalisation.
__global__ void mk_prop_crop_kernel(const float2 *__restrict__ G, int ny2, int nz2, int y0, int z0,
                                    int ny, int nz, float scale, float2 *__restrict__ field,
                                    float *__restrict__ intensity)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= ny || y >= nz) return;
    const float2 g = G[(size_t)(y + z0) * ny2 + (x + y0)];
    const float2 v = make_float2(g.x * scale, g.y * scale);
    if (field) field[(size_t)y * ny + x] = v;
    if (intensity) intensity[(size_t)y * ny + x] = v.x * v.x + v.y * v.y;
}

// ------------------------------------------------ fused spectral row pass
// The 2-D transform separates into a transform along z (columns) and one
// along y (rows), in either order. Taking the columns first and last,
//   G = C^-1 R^-1 [H o (R C P)] = C^-1 (R^-1 H R) C P,
// the row transform, the transfer-function multiply and the inverse row
// transform are adjacent: one kernel does all three per row in shared
// memory, so the spectrum is read and written once between the two column
// transforms (cuFFT) instead of three times (row FFT, multiply, inverse row
// FFT).
//
// Row FFT: Stockham autosort passes of radix 8 (then 4 or 2 for the rest of
// log2 N) between two shared-memory rows. Twiddles come from a table of exp(-2 pi i t / N) made in FP64
// (mk_prop_twiddles). The transfer function is formed in FP32 as the
// reference's prop_mul_kernel does (Beam.py:4763-4830), with the two large
// constant phases, z (k - k_axis) and -z k_axis, reduced mod 2 pi in FP64 on
// the host.
#define MK_FFT_NT 512
#define MK_FFT_MAX 8192

__device__ __forceinline__ float2 mk_cmul(float2 a, float2 b)
{
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

// In-register DFT of R = 2, 4, 8 points (natural order in and out); INV
// uses exp(+i ...).
template <int R, bool INV>
__device__ __forceinline__ void mk_dft(float2 (&v)[R])
{
    if constexpr (R == 2) {
        const float2 a = v[0], b = v[1];
        v[0] = make_float2(a.x + b.x, a.y + b.y);
        v[1] = make_float2(a.x - b.x, a.y - b.y);
    } else if constexpr (R == 4) {
        const float2 a0 = make_float2(v[0].x + v[2].x, v[0].y + v[2].y);
        const float2 a1 = make_float2(v[0].x - v[2].x, v[0].y - v[2].y);
        const float2 b0 = make_float2(v[1].x + v[3].x, v[1].y + v[3].y);
        float2 b1 = make_float2(v[1].x - v[3].x, v[1].y - v[3].y);
        // b1 * (-i) forward, * (+i) inverse
        b1 = INV ? make_float2(-b1.y, b1.x) : make_float2(b1.y, -b1.x);
        v[0] = make_float2(a0.x + b0.x, a0.y + b0.y);
        v[2] = make_float2(a0.x - b0.x, a0.y - b0.y);
        v[1] = make_float2(a1.x + b1.x, a1.y + b1.y);
        v[3] = make_float2(a1.x - b1.x, a1.y - b1.y);
    } else {
        // 8 = 2 x 4: DFT-4 of the even and odd points, twiddle the odd ones
        // by exp(-/+ 2 pi i m / 8), combine
        float2 e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
        mk_dft<4, INV>(e);
        mk_dft<4, INV>(o);
        const float h = 0.70710678118654752f;
        const float sg = INV ? 1.f : -1.f;
        o[1] = mk_cmul(o[1], make_float2(h, sg * h));
        o[2] = INV ? make_float2(-o[2].y, o[2].x) : make_float2(o[2].y, -o[2].x);
        o[3] = mk_cmul(o[3], make_float2(-h, sg * h));
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            v[m] = make_float2(e[m].x + o[m].x, e[m].y + o[m].y);
            v[m + 4] = make_float2(e[m].x - o[m].x, e[m].y - o[m].y);
        }
    }
}

// One Stockham pass of radix R over a row of N points, from one shared-
// memory buffer to the other; Ns = product of the radices before it.
// Butterfly j reads points j + r N/R, twiddles them by
// exp(-/+ 2 pi i r (j mod Ns) / (Ns R)) and writes its R outputs to
// (j - j mod Ns) R + j mod Ns + r Ns.
template <int R, bool INV>
__device__ __forceinline__ void mk_fft_pass(const float2 *src, float2 *dst, int N, int Ns,
                                            const float2 *__restrict__ tw)
{
    const int nb = N / R;
    const int tstep = N / (Ns * R);
    for (int j = threadIdx.x; j < nb; j += MK_FFT_NT) {
        float2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = src[j + r * nb];
        const int k = j & (Ns - 1);
        if (Ns > 1) {
#pragma unroll
            for (int r = 1; r < R; ++r) {
                float2 w = __ldg(tw + r * k * tstep);
                if (INV) w.y = -w.y;
                v[r] = mk_cmul(v[r], w);
            }
        }
        mk_dft<R, INV>(v);
        const int base = (j - k) * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) dst[base + r * Ns] = v[r];
    }
    __syncthreads();
}

// FFT of the row in buf[0]; returns the buffer (0 or 1) holding the result.
template <bool INV>
__device__ __forceinline__ int mk_fft_row(float2 *buf0, float2 *buf1, int N, int logn,
                                          const float2 *__restrict__ tw)
{
    float2 *src = buf0, *dst = buf1;
    int Ns = 1, left = logn, at = 0;
    for (; left >= 3; left -= 3, Ns *= 8) {
        mk_fft_pass<8, INV>(src, dst, N, Ns, tw);
        float2 *t = src; src = dst; dst = t; at ^= 1;
    }
    if (left == 2) {
        mk_fft_pass<4, INV>(src, dst, N, Ns, tw);
        at ^= 1;
    } else if (left == 1) {
        mk_fft_pass<2, INV>(src, dst, N, Ns, tw);
        at ^= 1;
    }
    return at;
}

// F (nz2, ny2) column-transformed spectrum, in place: each row y-transformed,
// multiplied by H(ky[x], kz[row]) and inverse y-transformed (unnormalised).
// ky, kz: FP32 transverse wavenumbers (2 pi fftfreq + carrier offset) of
// every column and row; c_prop = z (k - k_axis) mod 2 pi, c_evan =
// -z k_axis mod 2 pi. Shared memory: two rows (ping-pong between passes).
__global__ void __launch_bounds__(MK_FFT_NT)
    mk_prop_rows_kernel(float2 *__restrict__ F, int ny2, int logn, int nz2,
                        const float2 *__restrict__ tw, const float *__restrict__ ky,
                        const float *__restrict__ kz, float k, float z, float c_prop, float c_evan)
{
    extern __shared__ __align__(16) float2 s_buf[];
    float2 *b0 = s_buf, *b1 = s_buf + ny2;
    for (int rowi = blockIdx.x; rowi < nz2; rowi += gridDim.x) {
        float2 *g = F + (size_t)rowi * ny2;
        for (int x = threadIdx.x; x < ny2; x += MK_FFT_NT) b0[x] = g[x];
        __syncthreads();
        float2 *spec = mk_fft_row<false>(b0, b1, ny2, logn, tw) ? b1 : b0;
        const float b = kz[rowi];
        for (int x = threadIdx.x; x < ny2; x += MK_FFT_NT) {
            const float a = ky[x];
            const float kt2 = fmaf(a, a, b * b);
            const float kt = sqrtf(kt2);
            float ph, amp;
            if (kt <= k) {
                // sqrt(k^2 - kt^2) - k = -kt^2 / (sqrt(k^2 - kt^2) + k)
                ph = -z * kt2 / (sqrtf((k - kt) * (k + kt)) + k) + c_prop;
                amp = 1.f;
            } else {
                amp = expf(-fabsf(z) * sqrtf((kt - k) * (kt + k)));
                ph = c_evan;
            }
            float sn, cs;
            sincosf(ph, &sn, &cs);
            b0[x] = mk_cmul(spec[x], make_float2(amp * cs, amp * sn));
        }
        __syncthreads();
        const float2 *res = mk_fft_row<true>(b0, b1, ny2, logn, tw) ? b1 : b0;
        for (int x = threadIdx.x; x < ny2; x += MK_FFT_NT) g[x] = res[x];
        __syncthreads();
    }
}

// exp(-2 pi i t / n), t < n, from FP64 sincospi.
__global__ void mk_prop_twiddle_kernel(float2 *__restrict__ tw, int n)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    double s, c;
    sincospi(-2.0 * (double)t / (double)n, &s, &c);
    tw[t] = make_float2((float)c, (float)s);
}

// 2 pi fftfreq(n, d) + off as float32 (numpy ordering), in FP64.
__global__ void mk_prop_freq_kernel(float *__restrict__ out, int n, double d, double off)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = (float)(MK_TWO_PI * mk_fftfreq(i, n, d) + off);
}

extern "C" size_t mk_prop_rows_workspace_size(int ny2, int nz2)
{
    if (ny2 <= 0 || nz2 <= 0) return 0;
    return sizeof(float2) * (size_t)ny2 + sizeof(float) * ((size_t)ny2 + (size_t)nz2) + 256;
}

extern "C" int mk_prop_rows(float *spectrum, int ny2, int nz2, double dy, double dz, double k,
                            double z, double k_axis, double k_perp_y, double k_perp_z,
                            void *workspace, size_t ws_bytes, void *stream)
{
    MK_REQUIRE(spectrum && ny2 > 0 && nz2 > 0 && dy > 0.0 && dz > 0.0 && k > 0.0,
               "mk_prop_rows: bad arguments");
    MK_REQUIRE((ny2 & (ny2 - 1)) == 0 && ny2 >= 2 && ny2 <= MK_FFT_MAX,
               "mk_prop_rows: the row length %d must be a power of two in [2, %d]", ny2, MK_FFT_MAX);
    const size_t need = mk_prop_rows_workspace_size(ny2, nz2);
    if (!workspace || ws_bytes < need) {
        mk_set_error("mk_prop_rows: workspace %zu bytes, need %zu", ws_bytes, need);
        return MK_ENOMEM;
    }
    MK_REQUIRE(((uintptr_t)workspace & 15) == 0, "mk_prop_rows: workspace must be 16-byte aligned");
    int logn = 0;
    while ((1 << logn) < ny2) ++logn;
    cudaStream_t st = mk_stream(stream);
    float2 *tw = reinterpret_cast<float2 *>(workspace);
    float *ky = reinterpret_cast<float *>(tw + ny2);
    float *kz = ky + ny2;
    mk_prop_twiddle_kernel<<<(ny2 + 255) / 256, 256, 0, st>>>(tw, ny2);
    MK_CHECK_CUDA(cudaGetLastError());
    mk_prop_freq_kernel<<<(ny2 + 255) / 256, 256, 0, st>>>(ky, ny2, dy, k_perp_y);
    MK_CHECK_CUDA(cudaGetLastError());
    mk_prop_freq_kernel<<<(nz2 + 255) / 256, 256, 0, st>>>(kz, nz2, dz, k_perp_z);
    MK_CHECK_CUDA(cudaGetLastError());
    const double c_prop = fmod(z * (k - k_axis), MK_TWO_PI);
    const double c_evan = fmod(-z * k_axis, MK_TWO_PI);
    const size_t smem = 2 * sizeof(float2) * (size_t)ny2;
    MK_CHECK_CUDA(cudaFuncSetAttribute((const void *)mk_prop_rows_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int dev = 0, sms = 0, bps = 0;
    MK_CHECK_CUDA(cudaGetDevice(&dev));
    MK_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    MK_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, (const void *)mk_prop_rows_kernel,
                                                                MK_FFT_NT, smem));
    MK_REQUIRE(bps >= 1, "mk_prop_rows: a row of %d points does not fit on an SM", ny2);
    const int grid = std::min(nz2, sms * bps);
    mk_prop_rows_kernel<<<grid, MK_FFT_NT, smem, st>>>(reinterpret_cast<float2 *>(spectrum), ny2, logn,
                                                      nz2, tw, ky, kz, (float)k, (float)z,
                                                      (float)c_prop, (float)c_evan);
    MK_CHECK_CUDA(cudaGetLastError());
    return MK_OK;
}

extern "C" int mk_prop_pad(const float *field, int ny, int nz, float *padded, int ny2, int nz2,
                           int y0, int z0, int mode, float cval_re, float cval_im, void *stream)
{
    MK_REQUIRE(field && padded && ny > 0 && nz > 0 && ny2 >= ny && nz2 >= nz,
               "mk_prop_pad: bad arguments");
    MK_REQUIRE(y0 >= 0 && z0 >= 0 && y0 + ny <= ny2 && z0 + nz <= nz2, "mk_prop_pad: bad offsets");
    MK_REQUIRE(mode == 0 || mode == 1, "mk_prop_pad: mode must be 0 (edge) or 1 (constant)");
    dim3 g((ny2 + 255) / 256, nz2);
    mk_prop_pad_kernel<<<g, 256, 0, mk_stream(stream)>>>(
        reinterpret_cast<const float2 *>(field), ny, nz, reinterpret_cast<float2 *>(padded), ny2,
        nz2, y0, z0, mode, make_float2(cval_re, cval_im));
    MK_CHECK_CUDA(cudaGetLastError());
    return MK_OK;
}

extern "C" int mk_prop_mul(float *spectrum, int ny2, int nz2, double dy, double dz, double k,
                           double z, double k_axis, double k_perp_y, double k_perp_z, void *stream)
{
    MK_REQUIRE(spectrum && ny2 > 0 && nz2 > 0 && dy > 0.0 && dz > 0.0 && k > 0.0,
               "mk_prop_mul: bad arguments");
    dim3 g((ny2 + 255) / 256, nz2);
    mk_prop_mul_kernel<<<g, 256, 0, mk_stream(stream)>>>(reinterpret_cast<float2 *>(spectrum), ny2,
                                                        nz2, dy, dz, k, z, k_axis, k_perp_y,
                                                        k_perp_z);
    MK_CHECK_CUDA(cudaGetLastError());
    return MK_OK;
}

extern "C" int mk_prop_crop_abs2(const float *grid, int ny2, int nz2, int y0, int z0, int ny,
                                 int nz, float scale, float *field, float *intensity, void *stream)
{
    MK_REQUIRE(grid && ny > 0 && nz > 0 && y0 >= 0 && z0 >= 0 && y0 + ny <= ny2 && z0 + nz <= nz2,
               "mk_prop_crop_abs2: bad arguments");
    MK_REQUIRE(field || intensity, "mk_prop_crop_abs2: nothing to write");
    dim3 g((ny + 255) / 256, nz);
    mk_prop_crop_kernel<<<g, 256, 0, mk_stream(stream)>>>(reinterpret_cast<const float2 *>(grid),
                                                         ny2, nz2, y0, z0, ny, nz, scale,
                                                         reinterpret_cast<float2 *>(field),
                                                         intensity);
    MK_CHECK_CUDA(cudaGetLastError());
    return MK_OK;
}
