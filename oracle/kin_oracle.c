/*
 * CPU oracle for the kinematic scattering sum -- TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load this library, and only as the checker or as the timed CPU baseline.
 * The product path (mosaic_gb300) never calls it.
 *
 * This is a plain-C, double-precision restatement of the reference CPU
 * kernel `compute_scattering_cffi` (MOSAIC Beam.py:663-816) with two
 * deliberate differences:
 *   - the accumulators are returned in double (the reference casts them to
 *     float32 once at the end, Beam.py:810-813);
 *   - an optional per-atom Debye-Waller B (A^2) multiplies the scattering
 *     factor by exp(-B s^2); the reference has no such term, and passing
 *     NULL reproduces it exactly.
 *
 * Per pixel P (metres) and atom a (metres), with a +x beam:
 *   r    = |P - a|, dotv = (P - a)_x / r          (cos 2theta)
 *   Q    = k sqrt(2 (1 - dotv)),  s = Q * 0.25e-10 / pi   (sin(theta)/lambda, 1/A)
 *   f    = f0_WK(s) + f' + i f''                   (Beam.py:669-679, 765-774)
 *          minus (f0(0) + f' + i f'') when remove_forward and Q < Q_cut(P)
 *   term = E_in(a) f exp(i fmod(k (a_x + r), 2 pi)) r_e [R0/r] [sqrt(P_pol)]
 * with Q_cut(P) from the right/up pixel neighbours (Beam.py:716-746) and the
 * polarization factor P_pol = (1-p)(1+dotv^2)/2 + p(1-(e.r_hat)^2) clamped to
 * [0,1] (Beam.py:793-801).
 *
 * Optional analyser (the reference's GPU general kernel only, Beam.py:2350-2378;
 * its CPU path ignores it): theta = angle between r_hat and the analyser axis
 * c, evaluated as theta = 2 asin(|r_hat - c| / 2); top-hat: term x 0 when
 * theta > alpha; Darwin: term x 1 / (1 + (theta / hw)^2) (x 1 when hw <= 0).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define MKO_TWO_PI 6.283185307179586
#define MKO_RE 2.81794092e-15 /* classical electron radius [m], Beam.py:704 */

/* Waasmaier-Kirfel f0 at s^2 = (sin(theta)/lambda)^2 [1/A^2]; p = a1..a5, c, b1..b5
 * (Beam.py:669-679). */
static double mko_f0(double s2, const float *p)
{
    double f = p[5];
    for (int i = 0; i < 5; ++i)
        f += (double)p[i] * exp(-(double)p[6 + i] * s2);
    return f;
}

/* Forward-removal cut-off Q_cut per pixel: half the pixel diagonal in Q from
 * the right and upper neighbours, edge pixels using the inner neighbour
 * (Beam.py:716-746). Pixel p sits at column p % ny, row p / ny. */
static void mko_qcut(int ny, int nz, const double *cx, const double *cy,
                     const double *cz, double k, double *qcut, double *r0)
{
    const int npix = ny * nz;
    for (int p = 0; p < npix; ++p) {
        const int col = p % ny, row = p / ny;
        const double tx = cx[p], ty = cy[p], tz = cz[p];
        const double R0 = sqrt(tx * tx + ty * ty + tz * tz);
        double ux = 0.0, uy = 0.0, uz = 0.0;
        r0[p] = R0;
        if (R0 > 0.0) { ux = tx / R0; uy = ty / R0; uz = tz / R0; }
        const int nb[2] = {
            (col + 1 < ny) ? p + 1 : ((col > 0) ? p - 1 : p),
            (row + 1 < nz) ? p + ny : ((row > 0) ? p - ny : p)};
        double q[2];
        for (int j = 0; j < 2; ++j) {
            const double rx = cx[nb[j]], ry = cy[nb[j]], rz = cz[nb[j]];
            const double Rr = sqrt(rx * rx + ry * ry + rz * rz);
            double c = (Rr > 0.0) ? (ux * rx + uy * ry + uz * rz) / Rr : 1.0;
            if (c > 1.0) c = 1.0;
            if (c < -1.0) c = -1.0;
            const double d = 2.0 * (1.0 - c);
            q[j] = k * sqrt(d > 0.0 ? d : 0.0);
        }
        qcut[p] = 0.5 * sqrt(q[0] * q[0] + q[1] * q[1]);
    }
}

typedef struct {
    int64_t a0, a1;
    const double *pos;
    const float *wk, *f0z, *anr, *ani, *ampr, *ampi, *dwb;
    int remove_forward, apply_pol, decay;
    int npix;
    const double *cx, *cy, *cz, *qcut, *r0;
    double k, pdeg, ex, ey, ez;
    int analyser;
    double anx, any, anz, accept, hw;
    double *acc_r, *acc_i; /* this slice's own accumulators */
} mko_slice;

static void *mko_run_slice(void *arg)
{
    mko_slice *S = (mko_slice *)arg;
    const double s_fac = 0.25e-10 / 3.14159265358979323846;
    for (int64_t a = S->a0; a < S->a1; ++a) {
        const double ax = S->pos[3 * a], ay = S->pos[3 * a + 1], az = S->pos[3 * a + 2];
        const float *wk = S->wk + 11 * a;
        const double f00 = S->f0z[a], fr = S->anr[a], fi = S->ani[a];
        const double er = S->ampr[a], ei = S->ampi[a];
        const double B = S->dwb ? (double)S->dwb[a] : 0.0;
        for (int p = 0; p < S->npix; ++p) {
            const double dx = S->cx[p] - ax, dy = S->cy[p] - ay, dz = S->cz[p] - az;
            const double r = sqrt(dx * dx + dy * dy + dz * dz);
            if (r == 0.0) continue;
            const double dotv = dx / r;
            const double g = 2.0 * (1.0 - dotv);
            const double Q = S->k * sqrt(g > 0.0 ? g : 0.0);
            const double s = s_fac * Q, s2 = s * s;
            double fre = mko_f0(s2, wk) + fr, fim = fi;
            if (S->remove_forward && Q < S->qcut[p]) {
                fre -= (f00 + fr);
                fim -= fi;
            }
            if (B != 0.0) {
                const double w = exp(-B * s2);
                fre *= w; fim *= w;
            }
            const double tr = er * fre - ei * fim, ti = er * fim + ei * fre;
            const double ph = fmod(S->k * (ax + r), MKO_TWO_PI);
            const double c = cos(ph), sn = sin(ph);
            double scale = MKO_RE;
            if (S->decay && S->r0[p] > 0.0) scale *= S->r0[p] / r;
            if (S->apply_pol) {
                const double e = (S->ex * dx + S->ey * dy + S->ez * dz) / r;
                double P = 0.5 * (1.0 - S->pdeg) * (1.0 + dotv * dotv) + S->pdeg * (1.0 - e * e);
                if (P < 0.0) P = 0.0;
                if (P > 1.0) P = 1.0;
                scale *= sqrt(P);
            }
            if (S->analyser) {
                const double vx = dx / r - S->anx, vy = dy / r - S->any, vz = dz / r - S->anz;
                const double th = 2.0 * asin(0.5 * sqrt(vx * vx + vy * vy + vz * vz));
                if (S->analyser == 1) {
                    if (th > S->accept) scale = 0.0;
                } else if (S->analyser == 2 && S->hw > 0.0) {
                    const double t = th / S->hw;
                    scale *= 1.0 / (1.0 + t * t);
                }
            }
            S->acc_r[p] += (tr * c - ti * sn) * scale;
            S->acc_i[p] += (tr * sn + ti * c) * scale;
        }
    }
    return NULL;
}

/*
 * The FP64 sum, added into out_re/out_im (double, length ny*nz).
 * Atoms are split into n_threads contiguous slices; each slice sums into its
 * own buffers, which are then added in slice order, so the result does not
 * depend on thread timing (the reference sums its slices in submission order,
 * Beam.py:5941-5955). Returns 0, or 1 when a work buffer cannot be allocated
 * (the reference's MemoryError path, Beam.py:5768-5769).
 */
int mko_scatter_f64(int64_t n_atoms, const double *pos, const float *wk,
                    const float *f0z, int remove_forward, const float *anom_re,
                    const float *anom_im, const float *amp_re, const float *amp_im,
                    const float *dw_b, int ny, int nz, const double *cx,
                    const double *cy, const double *cz, double k, int apply_pol,
                    double pol_deg, double pol_ex, double pol_ey, double pol_ez,
                    int decay, int analyser, const double *an_axis, double an_accept,
                    double an_halfwidth, double *out_re, double *out_im, int n_threads)
{
    const int npix = ny * nz;
    if (n_atoms <= 0 || npix <= 0) return 0;
    if (n_threads < 1) n_threads = 1;
    if ((int64_t)n_threads > n_atoms) n_threads = (int)n_atoms;

    double *qcut = (double *)malloc((size_t)npix * sizeof(double));
    double *r0 = (double *)malloc((size_t)npix * sizeof(double));
    double *acc = (double *)calloc((size_t)npix * 2 * (size_t)n_threads, sizeof(double));
    mko_slice *sl = (mko_slice *)calloc((size_t)n_threads, sizeof(mko_slice));
    pthread_t *th = (pthread_t *)calloc((size_t)n_threads, sizeof(pthread_t));
    if (!qcut || !r0 || !acc || !sl || !th) {
        free(qcut); free(r0); free(acc); free(sl); free(th);
        return 1;
    }
    mko_qcut(ny, nz, cx, cy, cz, k, qcut, r0);

    const int64_t per = (n_atoms + n_threads - 1) / n_threads;
    for (int t = 0; t < n_threads; ++t) {
        mko_slice *S = &sl[t];
        S->a0 = (int64_t)t * per;
        S->a1 = S->a0 + per < n_atoms ? S->a0 + per : n_atoms;
        S->pos = pos; S->wk = wk; S->f0z = f0z; S->anr = anom_re; S->ani = anom_im;
        S->ampr = amp_re; S->ampi = amp_im; S->dwb = dw_b;
        S->remove_forward = remove_forward; S->apply_pol = apply_pol; S->decay = decay;
        S->npix = npix; S->cx = cx; S->cy = cy; S->cz = cz; S->qcut = qcut; S->r0 = r0;
        S->k = k; S->pdeg = pol_deg; S->ex = pol_ex; S->ey = pol_ey; S->ez = pol_ez;
        S->analyser = analyser;
        if (analyser) {
            const double n = sqrt(an_axis[0] * an_axis[0] + an_axis[1] * an_axis[1] +
                                  an_axis[2] * an_axis[2]);
            S->anx = an_axis[0] / n; S->any = an_axis[1] / n; S->anz = an_axis[2] / n;
        }
        S->accept = an_accept; S->hw = an_halfwidth;
        S->acc_r = acc + (size_t)2 * npix * t;
        S->acc_i = S->acc_r + npix;
    }
    int started = 0;
    for (int t = 1; t < n_threads; ++t) {
        if (pthread_create(&th[t], NULL, mko_run_slice, &sl[t]) != 0) break;
        started = t;
    }
    mko_run_slice(&sl[0]);
    for (int t = 1; t <= started; ++t) pthread_join(th[t], NULL);
    for (int t = started + 1; t < n_threads; ++t) mko_run_slice(&sl[t]);

    for (int t = 0; t < n_threads; ++t) {
        const double *ar = sl[t].acc_r, *ai = sl[t].acc_i;
        for (int p = 0; p < npix; ++p) { out_re[p] += ar[p]; out_im[p] += ai[p]; }
    }
    free(qcut); free(r0); free(acc); free(sl); free(th);
    return 0;
}

/*
 * Free-space propagator multiply, restated in double from the reference
 * `prop_mul_kernel` / `prop_mul_cpu` (Beam.py:4747-4834, 4849-4888):
 *   propagating (k^2 >= kt^2): H = exp(i [ -z kt^2/(sqrt(k^2-kt^2)+k) + z (k - kga) ])
 *   evanescent:                H = exp(-|z| sqrt(kt^2-k^2)) exp(-i z kga)
 * with kt = (ky + kgy, kz + kgz). F is the (nz, ny) spectrum, interleaved re/im,
 * multiplied in place.
 */
void mko_prop_mul_f64(int ny, int nz, const double *ky, const double *kz, double k,
                      double z, double kga, double kgy, double kgz, double *F)
{
    for (int iz = 0; iz < nz; ++iz) {
        for (int iy = 0; iy < ny; ++iy) {
            const double a = ky[iy] + kgy, b = kz[iz] + kgz;
            const double kt2 = a * a + b * b, kx2 = k * k - kt2;
            double ph, amp;
            if (kx2 >= 0.0) {
                ph = -z * kt2 / (sqrt(kx2) + k) + z * (k - kga);
                amp = 1.0;
            } else {
                amp = exp(-fabs(z) * sqrt(-kx2));
                ph = -z * kga;
            }
            const double hr = amp * cos(ph), hi = amp * sin(ph);
            double *g = F + 2 * ((size_t)iz * ny + iy);
            const double gr = g[0], gi = g[1];
            g[0] = gr * hr - gi * hi;
            g[1] = gr * hi + gi * hr;
        }
    }
}
