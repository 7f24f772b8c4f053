// Depth-dependent incident field (MOSAIC Beam.py:956-1045, 4963-5140,
// 5583-5618, 7118-7283): the sample's transmission map A(u, v) on the beam
// grid from the forward scattering factors of all atoms, and the per-atom
// amplitude E0 exp(-f tau) exp(i f phi) with f the atom's depth fraction
// along the beam.
//
// Arithmetic follows the reference's float32 order with explicit rounding
// intrinsics (no contraction): the map is a sum of triangular-shaped-cloud
// deposits (float atomics, so only the order of the additions differs from
// the reference's sequential np.add.at), and the per-atom field is the same
// sequence of float32 operations as the reference's NumPy code.
#include "mk_common.cuh"

// Triangular-shaped-cloud weight at distance d (grid units), evaluated in
// double and rounded once to float as the reference stores it.
__device__ __forceinline__ float mk_tsc(double d)
{
    if (d <= 0.5) return (float)(0.75 - d * d);
    if (d <= 1.5) {
        const double t = 1.5 - d;
        return (float)(0.5 * t * t);
    }
    return 0.f;
}

// The float32 lab position [A] that mk_atoms_lab divided by 1e10: the double
// quotient times 1e10 is within two double ulps of it, so the cast recovers it.
__device__ __forceinline__ float mk_lab_A(double m) { return (float)(m * 1e10); }

__global__ void mk_column_deposit_kernel(int64_t n, const double *__restrict__ pos,
                                         const int *__restrict__ species,
                                         const float2 *__restrict__ fwd, int ny, int nz,
                                         double du, double dv, double uc, double vc,
                                         float *__restrict__ sr, float *__restrict__ si)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // +x beam: the transverse basis is (y, z)
    const double iu = (double)mk_lab_A(pos[3 * i + 1]) / du + uc;
    const double iv = (double)mk_lab_A(pos[3 * i + 2]) / dv + vc;
    if (!(iu >= 0.0 && iu <= (double)(ny - 1) && iv >= 0.0 && iv <= (double)(nz - 1))) return;
    const float2 f = fwd[species[i]];
    const long long ic = (long long)floor(iu + 0.5), jc = (long long)floor(iv + 0.5);
#pragma unroll
    for (int dx = -1; dx <= 1; ++dx) {
        const long long ii = ic + dx;
        const float wx = mk_tsc(fabs(iu - (double)ii));
#pragma unroll
        for (int dy = -1; dy <= 1; ++dy) {
            const long long jj = jc + dy;
            const float fac = __fmul_rn(wx, mk_tsc(fabs(iv - (double)jj)));
            if (ii < 0 || ii >= ny || jj < 0 || jj >= nz || !(fac > 0.f)) continue;
            atomicAdd(&sr[ii * nz + jj], __fmul_rn(f.x, fac));
            atomicAdd(&si[ii * nz + jj], __fmul_rn(f.y, fac));
        }
    }
}

extern "C" int mk_beam_column_sums(int64_t n, const double *pos_lab, const int *species,
                                   const float *fwd, int n_species, int grid_ny, int grid_nz,
                                   const double *grid, float *sum_re, float *sum_im, void *stream)
{
    MK_REQUIRE(n >= 0 && grid_ny > 0 && grid_nz > 0 && grid && sum_re && sum_im,
               "mk_beam_column_sums: bad arguments");
    MK_REQUIRE(grid[0] > 0.0 && grid[1] > 0.0, "mk_beam_column_sums: grid spacings must be positive");
    MK_REQUIRE(n == 0 || (pos_lab && species && fwd && n_species >= 1),
               "mk_beam_column_sums: null atom buffer");
    cudaStream_t st = mk_stream(stream);
    const size_t m = (size_t)grid_ny * grid_nz;
    MK_CHECK_CUDA(cudaMemsetAsync(sum_re, 0, m * sizeof(float), st));
    MK_CHECK_CUDA(cudaMemsetAsync(sum_im, 0, m * sizeof(float), st));
    if (n == 0) return MK_OK;
    const int th = 256;
    mk_column_deposit_kernel<<<(unsigned)((n + th - 1) / th), th, 0, st>>>(
        n, pos_lab, species, reinterpret_cast<const float2 *>(fwd), grid_ny, grid_nz, grid[0],
        grid[1], grid[2], grid[3], sum_re, sum_im);
    MK_CHECK_CUDA(cudaGetLastError());
    return MK_OK;
}

// Column sums -> phase and attenuation: delta, beta = C x sums,
// phi = -k delta, tau = max(k beta, 0) (float32, constants rounded to float
// as the reference's NumPy expressions round them).
__global__ void mk_column_maps_kernel(int m, const float *__restrict__ sr,
                                      const float *__restrict__ si, float C, float k,
                                      float *__restrict__ tau, float *__restrict__ phi)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const float d = __fmul_rn(C, sr[i]);
    const float b = __fmul_rn(C, si[i]);
    phi[i] = __fmul_rn(-k, d);
    tau[i] = fmaxf(__fmul_rn(k, b), 0.f);
}

extern "C" int mk_beam_column_maps(int grid_ny, int grid_nz, const float *sum_re,
                                   const float *sum_im, double wavelength_A, double du_A,
                                   double dv_A, float *tau, float *phi, void *stream)
{
    MK_REQUIRE(grid_ny > 0 && grid_nz > 0 && sum_re && sum_im && tau && phi,
               "mk_beam_column_maps: bad arguments");
    MK_REQUIRE(wavelength_A > 0.0 && du_A > 0.0 && dv_A > 0.0,
               "mk_beam_column_maps: wavelength and spacings must be positive");
    const double r_e_A = MK_R_E * 1e10;
    const double C = r_e_A * wavelength_A * wavelength_A / (MK_TWO_PI * du_A * dv_A);
    const double k = MK_TWO_PI / wavelength_A;
    const int m = grid_ny * grid_nz;
    mk_column_maps_kernel<<<(m + 255) / 256, 256, 0, mk_stream(stream)>>>(m, sum_re, sum_im,
                                                                           (float)C, (float)k,
                                                                           tau, phi);
    MK_CHECK_CUDA(cudaGetLastError());
    return MK_OK;
}

// tau, phi as the per-atom field reads them: through the complex64 map
// A = exp(-tau + i phi), i.e. tau' = -log(|A| + 1e-20), phi' = arg A (wrapped).
__global__ void mk_column_wrap_kernel(int m, float *__restrict__ tau, float *__restrict__ phi)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const float e = expf(-tau[i]);
    float s, c;
    sincosf(phi[i], &s, &c);
    const float ar = __fmul_rn(e, c), ai = __fmul_rn(e, s);
    tau[i] = -logf(__fadd_rn(hypotf(ar, ai), 1e-20f));
    phi[i] = atan2f(ai, ar);
}

extern "C" int mk_beam_column_wrap(int grid_ny, int grid_nz, float *tau, float *phi, void *stream)
{
    MK_REQUIRE(grid_ny > 0 && grid_nz > 0 && tau && phi, "mk_beam_column_wrap: bad arguments");
    const int m = grid_ny * grid_nz;
    mk_column_wrap_kernel<<<(m + 255) / 256, 256, 0, mk_stream(stream)>>>(m, tau, phi);
    MK_CHECK_CUDA(cudaGetLastError());
    return MK_OK;
}

// Per-atom amplitude with the depth-dependent transmission (the reference's
// _ein_bilinear_cpu, term for term in float32).
__global__ void mk_ein_depth_kernel(int64_t n, const double *__restrict__ pos,
                                    const float2 *__restrict__ e0, const float *__restrict__ tau,
                                    const float *__restrict__ phi, int gny, int gnz, float du,
                                    float dv, float uc, float vc, float s_min, float denom,
                                    float2 *__restrict__ amp)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x = mk_lab_A(pos[3 * i]), y = mk_lab_A(pos[3 * i + 1]), z = mk_lab_A(pos[3 * i + 2]);
    const float iu = __fadd_rn(__fdiv_rn(y, du), uc);
    const float iv = __fadd_rn(__fdiv_rn(z, dv), vc);
    float2 a = make_float2(0.f, 0.f);
    if (iu >= 0.f && iu <= (float)(gny - 1) && iv >= 0.f && iv <= (float)(gnz - 1)) {
        const int i0 = (int)floorf(iu), j0 = (int)floorf(iv);
        const int i1 = min(i0 + 1, gny - 1), j1 = min(j0 + 1, gnz - 1);
        const float fu = __fsub_rn(iu, (float)i0), fv = __fsub_rn(iv, (float)j0);
        const float gu = __fsub_rn(1.f, fu), gv = __fsub_rn(1.f, fv);
        const float w00 = __fmul_rn(gu, gv), w01 = __fmul_rn(gu, fv);
        const float w10 = __fmul_rn(fu, gv), w11 = __fmul_rn(fu, fv);
        const int r00 = i0 * gnz + j0, r01 = i0 * gnz + j1, r10 = i1 * gnz + j0, r11 = i1 * gnz + j1;
        const float ts = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(tau[r00], w00), __fmul_rn(tau[r01], w01)),
                                             __fmul_rn(tau[r10], w10)),
                                   __fmul_rn(tau[r11], w11));
        const float ps = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(phi[r00], w00), __fmul_rn(phi[r01], w01)),
                                             __fmul_rn(phi[r10], w10)),
                                   __fmul_rn(phi[r11], w11));
        float er = 1.f, ei = 0.f;
        if (e0) {
            const float2 e00 = e0[r00], e01 = e0[r01], e10 = e0[r10], e11 = e0[r11];
            er = __fmul_rn(e00.x, w00);
            ei = __fmul_rn(e00.y, w00);
            er = __fadd_rn(er, __fmul_rn(e01.x, w01));
            ei = __fadd_rn(ei, __fmul_rn(e01.y, w01));
            er = __fadd_rn(er, __fmul_rn(e10.x, w10));
            ei = __fadd_rn(ei, __fmul_rn(e10.y, w10));
            er = __fadd_rn(er, __fmul_rn(e11.x, w11));
            ei = __fadd_rn(ei, __fmul_rn(e11.y, w11));
        }
        float f = __fdiv_rn(__fsub_rn(x, s_min), denom);
        f = fminf(fmaxf(f, 0.f), 1.f);
        const float at = expf(-__fmul_rn(f, ts));
        float sp, cp;
        sincosf(__fmul_rn(f, ps), &sp, &cp);
        const float re = __fmul_rn(__fsub_rn(__fmul_rn(er, cp), __fmul_rn(ei, sp)), at);
        const float im = __fmul_rn(__fadd_rn(__fmul_rn(er, sp), __fmul_rn(ei, cp)), at);
        a = make_float2(re, im);
    }
    amp[i] = a;
}

extern "C" int mk_atoms_ein_depth(int64_t n, const double *pos_lab, const float *e0,
                                  const float *tau, const float *phi, int grid_ny, int grid_nz,
                                  const double *grid, double s_min, double s_max, float *amp,
                                  void *stream)
{
    MK_REQUIRE(n >= 0, "mk_atoms_ein_depth: negative atom count");
    if (n == 0) return MK_OK;
    MK_REQUIRE(pos_lab && tau && phi && grid && amp, "mk_atoms_ein_depth: null argument");
    MK_REQUIRE(grid_ny > 0 && grid_nz > 0 && grid[0] > 0.0 && grid[1] > 0.0,
               "mk_atoms_ein_depth: beam grid needs positive sizes and spacings");
    double denom = s_max - s_min;
    if (!(denom > 0.0)) denom = 1.0;    // zero-thickness window (Beam.py:1027-1029)
    const int th = 256;
    mk_ein_depth_kernel<<<(unsigned)((n + th - 1) / th), th, 0, mk_stream(stream)>>>(
        n, pos_lab, reinterpret_cast<const float2 *>(e0), tau, phi, grid_ny, grid_nz,
        (float)grid[0], (float)grid[1], (float)grid[2], (float)grid[3], (float)s_min,
        (float)denom, reinterpret_cast<float2 *>(amp));
    MK_CHECK_CUDA(cudaGetLastError());
    return MK_OK;
}
