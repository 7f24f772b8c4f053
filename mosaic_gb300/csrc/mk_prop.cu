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
