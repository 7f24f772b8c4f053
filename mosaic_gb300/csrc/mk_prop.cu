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

// --------------------------------------------- fused spectral column pass
// The 2-D transform separates into a transform along y (rows) and one along
// z (columns), in either order. Taking the rows first and last,
//   G = R^-1 C^-1 [H o (C R P)] = R^-1 (C^-1 H C) R P,
// the column transform, the transfer-function multiply and the inverse
// column transform are adjacent: one kernel does all three for a group of
// W neighbouring columns in shared memory, so between the two row
// transforms (cuFFT, contiguous rows) the spectrum is read and written once
// instead of three times (column FFT, multiply, inverse column FFT).
//
// A block loads W columns (each row's W neighbours are one contiguous
// segment of 8 W bytes) into shared memory as W lines of N points in
// bit-reversed order (stride N + 1, which spreads a row's W points over
// different banks), transforms every line in place by radix-2
// decimation-in-time stages fused three at a time (a butterfly keeps its 8
// points in registers through the three stages and writes them back where
// it read them), applies H in natural order, bit-reverses the lines and
// transforms them back the same way, and writes the columns back. Twiddles come from a table of exp(-2 pi i t / N)
// made in FP64. The transfer function is formed in FP32 as the reference's
// prop_mul_kernel does (Beam.py:4763-4830), with the two large constant
// phases, z (k - k_axis) and -z k_axis, reduced mod 2 pi in FP64 on the
// host.
#define MK_FFT_NT 512
#define MK_FFT_MAX 8192
#define MK_FFT_PTS 16384          // W x N points a block holds

__device__ __forceinline__ float2 mk_cmul(float2 a, float2 b)
{
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

// Bit reversal of the low `bits` bits of i.
__device__ __forceinline__ int mk_bitrev(int i, int bits)
{
    return (int)(__brev((unsigned)i) >> (32 - bits));
}

// G consecutive in-place radix-2 decimation-in-time stages (half sizes m,
// 2m, .., 2^(G-1) m) fused into one pass over W lines of N points in shared
// memory (line c at s + c * ld; the lines were loaded in bit-reversed
// order). A butterfly owns the R = 2^G points b + i + r m (b a multiple of
// R m, i < m), keeps them in registers through the G stages and writes them
// back where it read them, so the pass works in place. Stage h pairs points
// a and a + 2^h (bit h of a clear) with the twiddle
// exp(-/+ 2 pi i j / (2^(h+1) m)), j = i + (a mod 2^h) m.
template <int G, bool INV>
__device__ __forceinline__ void mk_dit_pass(float2 *s, int ld, int W, int N, int m,
                                            const float2 *__restrict__ tw)
{
    constexpr int R = 1 << G;
    const int nb = N / R, total = W * nb;
    for (int t = threadIdx.x; t < total; t += MK_FFT_NT) {
        const int c = t / nb, q = t - c * nb;
        const int i = q & (m - 1);
        float2 *pts = s + c * ld + (q - i) * R + i;
        float2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = pts[r * m];
#pragma unroll
        for (int h = 0; h < G; ++h) {
            const int hs = m << h;
            const int tstep = N / (2 * hs);
#pragma unroll
            for (int a = 0; a < R; ++a) {
                if (a & (1 << h)) continue;
                const int j = i + (a & ((1 << h) - 1)) * m;
                float2 w = __ldg(tw + j * tstep);
                if (INV) w.y = -w.y;
                const float2 x = v[a], y = mk_cmul(v[a + (1 << h)], w);
                v[a] = make_float2(x.x + y.x, x.y + y.y);
                v[a + (1 << h)] = make_float2(x.x - y.x, x.y - y.y);
            }
        }
#pragma unroll
        for (int r = 0; r < R; ++r) pts[r * m] = v[r];
    }
    __syncthreads();
}

// FFT of W lines of N = 2^logn points loaded in bit-reversed order; the
// result is in natural order, in place.
template <bool INV>
__device__ __forceinline__ void mk_fft_lines(float2 *s, int ld, int W, int N, int logn,
                                             const float2 *__restrict__ tw)
{
    int m = 1, left = logn;
    for (; left >= 3; left -= 3, m <<= 3) mk_dit_pass<3, INV>(s, ld, W, N, m, tw);
    if (left == 2) mk_dit_pass<2, INV>(s, ld, W, N, m, tw);
    else if (left == 1) mk_dit_pass<1, INV>(s, ld, W, N, m, tw);
}

// In-place bit-reversal permutation of W lines (between the forward and the
// inverse transform, whose input must again be bit-reversed).
__device__ __forceinline__ void mk_bitrev_lines(float2 *s, int ld, int W, int N, int logn)
{
    for (int e = threadIdx.x; e < W * N; e += MK_FFT_NT) {
        const int c = e / N, r = e - c * N;
        const int q = mk_bitrev(r, logn);
        if (q > r) {
            float2 *line = s + c * ld;
            const float2 t = line[r];
            line[r] = line[q];
            line[q] = t;
        }
    }
    __syncthreads();
}

// F (nz2, ny2) row-transformed spectrum, in place: every column
// z-transformed, multiplied by H(ky[col], kz[row]) and inverse
// z-transformed (unnormalised). W columns a block; ky, kz: FP32 transverse
// wavenumbers (2 pi fftfreq + carrier offset) of every column and row;
// c_prop = z (k - k_axis) mod 2 pi, c_evan = -z k_axis mod 2 pi.
__global__ void __launch_bounds__(MK_FFT_NT)
    mk_prop_cols_kernel(float2 *__restrict__ F, int ny2, int nz2, int logn, int W,
                        const float2 *__restrict__ tw, const float *__restrict__ ky,
                        const float *__restrict__ kz, float k, float z, float c_prop, float c_evan)
{
    extern __shared__ __align__(16) float2 s_lines[];
    const int ld = nz2 + 1;
    const int groups = ny2 / W, pts = W * nz2;
    for (int g = blockIdx.x; g < groups; g += gridDim.x) {
        const int c0 = g * W;
        for (int e = threadIdx.x; e < pts; e += MK_FFT_NT) {
            const int r = e / W, c = e - r * W;
            s_lines[c * ld + mk_bitrev(r, logn)] = F[(size_t)r * ny2 + c0 + c];
        }
        __syncthreads();
        mk_fft_lines<false>(s_lines, ld, W, nz2, logn, tw);
        for (int e = threadIdx.x; e < pts; e += MK_FFT_NT) {
            const int c = e / nz2, r = e - c * nz2;
            const float a = ky[c0 + c], b = kz[r];
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
            float2 *p = s_lines + c * ld + r;
            *p = mk_cmul(*p, make_float2(amp * cs, amp * sn));
        }
        __syncthreads();
        mk_bitrev_lines(s_lines, ld, W, nz2, logn);
        mk_fft_lines<true>(s_lines, ld, W, nz2, logn, tw);
        for (int e = threadIdx.x; e < pts; e += MK_FFT_NT) {
            const int r = e / W, c = e - r * W;
            F[(size_t)r * ny2 + c0 + c] = s_lines[c * ld + r];
        }
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

// Columns a block: W x nz2 <= MK_FFT_PTS, at most 16 and the row length.
static int mk_prop_cols_width(int ny2, int nz2)
{
    int W = MK_FFT_PTS / nz2;
    W = std::min(W, 16);
    W = std::min(W, ny2);
    return std::max(W, 1);
}

extern "C" size_t mk_prop_cols_workspace_size(int ny2, int nz2)
{
    if (ny2 <= 0 || nz2 <= 0) return 0;
    return sizeof(float2) * (size_t)nz2 + sizeof(float) * ((size_t)ny2 + (size_t)nz2) + 256;
}

extern "C" int mk_prop_cols(float *spectrum, int ny2, int nz2, double dy, double dz, double k,
                            double z, double k_axis, double k_perp_y, double k_perp_z,
                            void *workspace, size_t ws_bytes, void *stream)
{
    MK_REQUIRE(spectrum && ny2 > 0 && nz2 > 0 && dy > 0.0 && dz > 0.0 && k > 0.0,
               "mk_prop_cols: bad arguments");
    MK_REQUIRE((nz2 & (nz2 - 1)) == 0 && nz2 >= 2 && nz2 <= MK_FFT_MAX,
               "mk_prop_cols: the column length %d must be a power of two in [2, %d]", nz2,
               MK_FFT_MAX);
    MK_REQUIRE((ny2 & (ny2 - 1)) == 0, "mk_prop_cols: the row length %d must be a power of two",
               ny2);
    const size_t need = mk_prop_cols_workspace_size(ny2, nz2);
    if (!workspace || ws_bytes < need) {
        mk_set_error("mk_prop_cols: workspace %zu bytes, need %zu", ws_bytes, need);
        return MK_ENOMEM;
    }
    MK_REQUIRE(((uintptr_t)workspace & 15) == 0, "mk_prop_cols: workspace must be 16-byte aligned");
    int logn = 0;
    while ((1 << logn) < nz2) ++logn;
    const int W = mk_prop_cols_width(ny2, nz2);
    cudaStream_t st = mk_stream(stream);
    float2 *tw = reinterpret_cast<float2 *>(workspace);
    float *ky = reinterpret_cast<float *>(tw + nz2);
    float *kz = ky + ny2;
    mk_prop_twiddle_kernel<<<(nz2 + 255) / 256, 256, 0, st>>>(tw, nz2);
    MK_CHECK_CUDA(cudaGetLastError());
    mk_prop_freq_kernel<<<(ny2 + 255) / 256, 256, 0, st>>>(ky, ny2, dy, k_perp_y);
    MK_CHECK_CUDA(cudaGetLastError());
    mk_prop_freq_kernel<<<(nz2 + 255) / 256, 256, 0, st>>>(kz, nz2, dz, k_perp_z);
    MK_CHECK_CUDA(cudaGetLastError());
    const double c_prop = fmod(z * (k - k_axis), MK_TWO_PI);
    const double c_evan = fmod(-z * k_axis, MK_TWO_PI);
    const size_t smem = sizeof(float2) * (size_t)W * (size_t)(nz2 + 1);
    MK_CHECK_CUDA(cudaFuncSetAttribute((const void *)mk_prop_cols_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int dev = 0, sms = 0, bps = 0;
    MK_CHECK_CUDA(cudaGetDevice(&dev));
    MK_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    MK_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, (const void *)mk_prop_cols_kernel,
                                                                MK_FFT_NT, smem));
    MK_REQUIRE(bps >= 1, "mk_prop_cols: %d columns of %d points do not fit on an SM", W, nz2);
    const int grid = std::min(ny2 / W, sms * bps);
    mk_prop_cols_kernel<<<grid, MK_FFT_NT, smem, st>>>(reinterpret_cast<float2 *>(spectrum), ny2, nz2,
                                                      logn, W, tw, ky, kz, (float)k, (float)z,
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
