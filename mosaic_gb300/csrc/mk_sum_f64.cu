// FP64 plain direct sum: the reference CPU kernel's arithmetic term for term
// (compute_scattering_cffi, MOSAIC Beam.py:748-808) on the GPU.
//
// This translation unit is compiled with --fmad=false so that, like the
// uncontracted C oracle, every product and sum rounds separately: the
// absolute phase k (x + r) is ~1e10 rad, where one double ulp is ~2e-6 rad,
// and a contracted build would differ from the CPU result at that level.
#include "mk_common.cuh"

int mk_launch_reduce(const double2 *partial, int slices, int n_pix, const double2 *phasor,
                     double scale, double2 *out, int accumulate, cudaStream_t st);

#define F64_NT 128
#define F64_ATOMS 128   // atoms staged in shared memory per step

// x mod y with the sign of x, exactly as C fmod: the remainder of two doubles
// is representable, so fma(-q, y, x) with the right integer quotient q
// returns it without rounding; q from the rounded division is corrected by
// one when it lands on the wrong side.
__device__ __forceinline__ double mk_fmod_exact(double x, double y)
{
    const double ax = fabs(x);
    if (ax < y) return x;
    double q = trunc(ax / y);
    double r = fma(-q, y, ax);
    if (r < 0.0) { q -= 1.0; r = fma(-q, y, ax); }
    else if (r >= y) { q += 1.0; r = fma(-q, y, ax); }
    return x < 0.0 ? -r : r;
}

struct MkPlainArgs {
    MkSpecies sp;
    double k;
    int apply_pol, decay, remove_forward;
    double pdeg, ex, ey, ez;
    int analyser;                      // 0 off, 1 top-hat, 2 Darwin
    double ax, ay, az, x_accept, hw;   // axis, 4 sin^2(alpha/2), half-width
};

__global__ void __launch_bounds__(F64_NT) mk_plain_f64_kernel(
    int64_t n, int64_t atoms_per_slice, const double *__restrict__ pos,
    const int *__restrict__ species, const float2 *__restrict__ amp, int n_pix,
    const double *__restrict__ xyz, const double *__restrict__ r0v,
    const double4 *__restrict__ qv, const __grid_constant__ MkPlainArgs A,
    double2 *__restrict__ partial)
{
    __shared__ double s_pos[F64_ATOMS][3];
    __shared__ int s_sp[F64_ATOMS];
    __shared__ float2 s_amp[F64_ATOMS];
    __shared__ float s_wk[MK_MAX_SPECIES][11];
    const int p = blockIdx.x * F64_NT + threadIdx.x;
    const bool live = p < n_pix;
    for (int i = threadIdx.x; i < MK_MAX_SPECIES * 11; i += F64_NT)
        s_wk[i / 11][i % 11] = A.sp.wk[i / 11][i % 11];
    const double cx = live ? xyz[3 * p] : 0.0, cy = live ? xyz[3 * p + 1] : 0.0,
                 cz = live ? xyz[3 * p + 2] : 0.0;
    const double R0 = live ? r0v[p] : 0.0, qcut = live ? qv[p].w : 0.0;
    const double s_fac = 0.25e-10 / MK_PI;
    double acc_r = 0.0, acc_i = 0.0;
    const int64_t a_lo = (int64_t)blockIdx.y * atoms_per_slice;
    const int64_t a_hi = min(n, a_lo + atoms_per_slice);
    for (int64_t a0 = a_lo; a0 < a_hi; a0 += F64_ATOMS) {
        const int m = (int)min((int64_t)F64_ATOMS, a_hi - a0);
        __syncthreads();
        for (int j = threadIdx.x; j < m; j += F64_NT) {
            s_pos[j][0] = pos[3 * (a0 + j)];
            s_pos[j][1] = pos[3 * (a0 + j) + 1];
            s_pos[j][2] = pos[3 * (a0 + j) + 2];
            s_sp[j] = species[a0 + j];
            s_amp[j] = amp[a0 + j];
        }
        __syncthreads();
        if (!live) continue;
        for (int j = 0; j < m; ++j) {
            const double ax = s_pos[j][0], ay = s_pos[j][1], az = s_pos[j][2];
            const int s = s_sp[j];
            const double dx = cx - ax, dy = cy - ay, dz = cz - az;
            const double r = sqrt(dx * dx + dy * dy + dz * dz);
            if (r == 0.0) continue;
            const double dotv = dx / r;
            const double g = 2.0 * (1.0 - dotv);
            const double Q = A.k * sqrt(g > 0.0 ? g : 0.0);
            const double sv = s_fac * Q, s2 = sv * sv;
            const float *wk = s_wk[s];
            double f0 = wk[5];
#pragma unroll
            for (int i = 0; i < 5; ++i) f0 += (double)wk[i] * exp(-(double)wk[6 + i] * s2);
            const double fr = A.sp.anr[s], fi = A.sp.ani[s];
            double fre = f0 + fr, fim = fi;
            if (A.remove_forward && Q < qcut) {
                fre -= ((double)A.sp.f0z[s] + fr);
                fim -= fi;
            }
            if (A.sp.has_dw) {
                const double B = A.sp.dwb[s];
                if (B != 0.0) {
                    const double w = exp(-B * s2);
                    fre *= w;
                    fim *= w;
                }
            }
            const double er = s_amp[j].x, ei = s_amp[j].y;
            const double tr = er * fre - ei * fim, ti = er * fim + ei * fre;
            const double ph = mk_fmod_exact(A.k * (ax + r), MK_TWO_PI);
            double sn, c;
            sincos(ph, &sn, &c);
            double scale = MK_R_E;
            if (A.decay && R0 > 0.0) scale *= R0 / r;
            if (A.apply_pol) {
                const double e = (A.ex * dx + A.ey * dy + A.ez * dz) / r;
                double P = 0.5 * (1.0 - A.pdeg) * (1.0 + dotv * dotv) + A.pdeg * (1.0 - e * e);
                P = P < 0.0 ? 0.0 : (P > 1.0 ? 1.0 : P);
                scale *= sqrt(P);
            }
            if (A.analyser) {
                const double vx = dx / r - A.ax, vy = dy / r - A.ay, vz = dz / r - A.az;
                scale *= mk_analyser_factor(A.analyser, vx * vx + vy * vy + vz * vz, A.x_accept,
                                            A.hw);
            }
            acc_r += (tr * c - ti * sn) * scale;
            acc_i += (tr * sn + ti * c) * scale;
        }
    }
    if (live) partial[(size_t)blockIdx.y * n_pix + p] = make_double2(acc_r, acc_i);
}

extern "C" size_t mk_sum_workspace_size(int n_pix, int slices)
{
    if (n_pix <= 0 || slices <= 0) return 256;
    return sizeof(double2) * (size_t)n_pix * (size_t)slices;
}

static int mk_plain_slices(int64_t n, int n_pix, int want)
{
    if (want > 0) return (int)std::min<int64_t>(want, std::max<int64_t>(1, (n + F64_ATOMS - 1) / F64_ATOMS));
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t bx = (n_pix + F64_NT - 1) / F64_NT;
    int64_t s = (8LL * sms + bx - 1) / bx;
    s = std::min<int64_t>(s, std::max<int64_t>(1, (n + 4 * F64_ATOMS - 1) / (4 * F64_ATOMS)));
    return (int)std::max<int64_t>(1, std::min<int64_t>(s, 4096));
}

extern "C" int mk_kin_plain_f64(int64_t n, const double *pos, const int *species,
                                const float *amp, const mk_species *spc, const mk_physics *phys,
                                const mk_pixels *px, int slices, double *out, int accumulate,
                                void *workspace, size_t ws_bytes, void *stream)
{
    MK_REQUIRE(spc && phys && px && out, "mk_kin_plain_f64: null argument");
    MK_REQUIRE(n >= 0, "mk_kin_plain_f64: negative atom count");
    const int64_t np64 = (int64_t)px->ny * px->nz;
    MK_REQUIRE(px->ny > 0 && px->nz > 0 && np64 < (1ll << 31), "mk_kin_plain_f64: bad detector shape");
    MK_REQUIRE(n == 0 || (pos && species && amp), "mk_kin_plain_f64: null atom buffer");
    MK_REQUIRE(px->xyz && px->r0 && px->q, "mk_kin_plain_f64: pixels not prepared");
    MK_REQUIRE(phys->k > 0.0, "mk_kin_plain_f64: k must be positive");
    const int n_pix = (int)np64;
    MkPlainArgs A;
    int rc = mk_species_pack(spc, &A.sp);
    if (rc != MK_OK) return rc;
    A.k = phys->k;
    A.apply_pol = phys->apply_pol;
    A.decay = phys->spherical_decay;
    A.remove_forward = phys->remove_forward;
    A.pdeg = phys->pol_deg;
    A.ex = phys->pol_e[0];
    A.ey = phys->pol_e[1];
    A.ez = phys->pol_e[2];
    rc = mk_analyser_pack(phys, &A.analyser, &A.ax, &A.ay, &A.az, &A.x_accept, &A.hw);
    if (rc != MK_OK) return rc;
    cudaStream_t st = mk_stream(stream);
    if (n == 0) {
        if (!accumulate) MK_CHECK_CUDA(cudaMemsetAsync(out, 0, sizeof(double2) * (size_t)n_pix, st));
        return MK_OK;
    }
    const int ns = mk_plain_slices(n, n_pix, slices);
    const size_t need = sizeof(double2) * (size_t)ns * n_pix;
    if (!workspace || ws_bytes < need) {
        mk_set_error("mk_kin_plain_f64: workspace %zu bytes, need %zu (slices=%d)", ws_bytes, need, ns);
        return MK_ENOMEM;
    }
    int64_t per = (n + ns - 1) / ns;
    per = ((per + F64_ATOMS - 1) / F64_ATOMS) * F64_ATOMS;
    const int ns_eff = (int)((n + per - 1) / per);
    dim3 grid((n_pix + F64_NT - 1) / F64_NT, ns_eff);
    double2 *part = static_cast<double2 *>(workspace);
    mk_plain_f64_kernel<<<grid, F64_NT, 0, st>>>(n, per, pos, species,
                                                 reinterpret_cast<const float2 *>(amp), n_pix,
                                                 px->xyz, px->r0,
                                                 reinterpret_cast<const double4 *>(px->q), A, part);
    MK_CHECK_CUDA(cudaGetLastError());
    return mk_launch_reduce(part, ns_eff, n_pix, nullptr, 1.0, reinterpret_cast<double2 *>(out),
                            accumulate, st);
}
