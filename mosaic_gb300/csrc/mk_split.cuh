// Device side of the FP32 split-phase kinematic sum: argument block,
// per-term loops and the persistent kernel template, included by the
// translation units that instantiate it (mk_split_k64/128/256.cu, one per
// block size, compiled in parallel) and by the host code (mk_sum_f32.cu).
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
// per-pixel vector q (from mk_pixels_prepare) with the FP64 tile origin,
// reduced mod 1 in FP64; the rest is small and FP32. Inside the tile the
// term phase is w.D (+ the |d|^2 term when `FRESNEL`), w = b - u', D the
// float32 offset in cycles: 3 FMA, a mod-1 reduction, and sin/cos on the MUFU.
//
// The direction-dependent factor (f0 + f' + i f'') exp(-B s^2) sqrt(P_pol)
// [R0/r] is evaluated once per (tile, pixel) at the tile direction u'; its
// change across a tile is ~|d|/|P| relative. Per-tile sums are folded into
// the per-pixel accumulators with Kahan compensation.
//
// Work decomposition: a frame (an exposure's pixels, or one scan step's ROI)
// is cut into pixel blocks (threads x pixels-per-thread) times tile slices;
// every (frame, pixel block, slice) is a work item. A persistent grid of
// one wave of blocks pulls items from an atomic counter, so frames of
// uneven size and the last partial wave cost no idle SMs. Each item writes
// its partial field; an FP64 pass adds the slices of every pixel in a fixed
// order, so the result does not depend on scheduling.
//
// Atom tiles reach shared memory by 1-D TMA bulk copies (cp.async.bulk),
// double-buffered on two mbarriers; every wait is bounded (mk_common.cuh).
#pragma once
#include <cuda_bf16.h>

#include "mk_common.cuh"

struct MkSplitArgs {
    MkSpecies sp;
    int n_tiles, tile_atoms, n_frames;
    long long n_items;
    mk_frame_desc f0;                // the frame when n_frames == 1
    const mk_frame_desc *frames;     // device, n_frames (n_frames > 1)
    unsigned long long *counter;
    const double4 *q;                // per pixel (qx, qy, qz, qcut)
    const float4 *u;                 // per pixel (ux, uy, uz, 1/|P|)
    const double4 *origin;
    const int *tspecies;
    const float4 *tpos;
    const float2 *tamp;
    double2 *partial;
    int *status;
    float kappa;       // k / 2 pi [cycles/m]
    float k;           // [1/m]
    float s2fac;       // (k 0.25e-10 / pi)^2: s^2 = s2fac |b - u'|^2 [1/A^2]
    int apply_pol, decay, remove_forward;
    float pdeg;
    float fres_r;      // tiles wider than this [m] keep the |d|^2 term (FRESNEL kernels)
    float pair_short_r; // pair/quad kernels: tiles up to this radius [m] use the short polynomials
    float sin_direct;   // quad kernels: in-tile phase bound [rad] below which the reduction is skipped
    float oct_r;        // octet / square kernels: tiles up to this radius [m] take that form, the rest quads
    // per-(species, pixel) factors at the pixel directions (mk_factor_table),
    // [species][ftab_n] float2, or null: the factor per (tile, pixel)
    const float2 *ftab;
    long long ftab_n;
    // analyser (ANA kernels, single exposures): kind 1 top-hat / 2 Darwin,
    // beam direction and analyser axis in FP64, 4 sin^2(alpha/2), half-width
    int analyser;
    double an_b[3], an_c[3];
    double an_xacc, an_hw, inv_kappa;
};

#define TWO_PI_F 6.28318530717958647692f
// 1.5 * 2^23: for |x| < 2^22, (x + C) - C is x rounded to the nearest
// integer (round-to-nearest-even of the FP32 add), two full-rate FMA-pipe
// adds instead of rintf, whose FRND shares the quarter-rate pipe with the
// MUFU sin/cos (measured 16 per clock per SM for each on sm_103).
#define MK_ROUND_MAGIC 12582912.0f

// x - nearest integer(x), exact in FP32 for |x| < 2^22.
__device__ __forceinline__ float mk_frac_nearest(float x)
{
    return __fsub_rn(x, __fsub_rn(__fadd_rn(x, MK_ROUND_MAGIC), MK_ROUND_MAGIC));
}

// Scattering factor of species s at direction u' = b - w.
__device__ __forceinline__ float2 mk_factor(const MkSplitArgs &A, int s, const mk_frame_desc &F,
                                           float wx, float wy, float wz, float qcut,
                                           float decay_ratio)
{
    const float upx = F.b[0] - wx, upy = F.b[1] - wy, upz = F.b[2] - wz;
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
        const float dotv = fmaf(F.b[2], upz, fmaf(F.b[1], upy, F.b[0] * upx));
        const float er = fmaf(F.e[2], upz, fmaf(F.e[1], upy, F.e[0] * upx));
        float P = 0.5f * (1.f - A.pdeg) * fmaf(dotv, dotv, 1.f) + A.pdeg * fmaf(-er, er, 1.f);
        P = fminf(1.f, fmaxf(0.f, P));
        scale *= sqrtf(P);
    }
    if (A.decay) scale *= decay_ratio;
    return make_float2(fr * scale, fi * scale);
}

__device__ __forceinline__ void mk_issue_tile(const MkSplitArgs &A, float4 *s_pos, float2 *s_amp,
                                              uint64_t *bar, int buf, int tile, int T,
                                              uint32_t tile_bytes)
{
    mk_mbar_expect_tx(&bar[buf], tile_bytes);
    mk_tma_load_1d(s_pos + buf * T, A.tpos + (size_t)tile * T, T * sizeof(float4), &bar[buf]);
    mk_tma_load_1d(s_amp + buf * T, A.tamp + (size_t)tile * T, T * sizeof(float2), &bar[buf]);
}

// A pixel's (u, 1/|P|) read again for the fold: an opaque load, so that the
// compiler rebuilds w there instead of keeping the values from before the
// atom loop live across it (registers the quad kernels need for occupancy).
__device__ __forceinline__ float4 mk_ld_fold(const float4 *p)
{
    float4 v;
    asm volatile("ld.global.nc.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p));
    return v;
}

// A tile's FP64 origin read again for the fold (opaque, like mk_ld_fold).
__device__ __forceinline__ double4 mk_ld_origin(const double4 *p)
{
    double4 v;
    asm volatile("ld.global.nc.v2.f64 {%0, %1}, [%4];\n\t"
                 "ld.global.nc.v2.f64 {%2, %3}, [%4+16];"
                 : "=d"(v.x), "=d"(v.y), "=d"(v.z), "=d"(v.w) : "l"(p));
    return v;
}

// Tile atoms in shared memory come in interleaved pairs (see mk_tiles_build):
// float4 P[2q] = (x0, x1, y0, y1), P[2q+1] = (z0, z1, w0, w1) and
// float4 E[q] = (re0, re1, im0, im1) for atoms 2q, 2q+1.
struct MkAtom {
    float4 a;   // x, y, z (cycles), |D|^2
    float2 e;   // amplitude
};
__device__ __forceinline__ void mk_atom_pair(const float4 *__restrict__ P,
                                             const float4 *__restrict__ E, int q, MkAtom &u,
                                             MkAtom &v)
{
    const float4 A = P[2 * q], B = P[2 * q + 1], M = E[q];
    u.a = make_float4(A.x, A.z, B.x, B.z);
    v.a = make_float4(A.y, A.w, B.y, B.w);
    u.e = make_float2(M.x, M.z);
    v.e = make_float2(M.y, M.w);
}

// The terms of one tile against PIX pixels: csr/csi += E_j exp(2 pi i phase).
// FR adds the |d|^2 term of the in-tile distance (db = D.b per atom).
template <int PIX, bool FR, bool CPLX>
__device__ __forceinline__ void mk_atom_terms(const MkAtom &at, const float (&wx)[PIX],
                                              const float (&wy)[PIX], const float (&wz)[PIX],
                                              const float (&hq)[PIX], float bx, float by,
                                              float bz, float (&csr)[PIX], float (&csi)[PIX])
{
    const float4 a = at.a;
    const float2 e = at.e;
    float db = 0.f;
    if (FR) db = fmaf(a.z, bz, fmaf(a.y, by, a.x * bx));
#pragma unroll
    for (int p = 0; p < PIX; ++p) {
        float lin = fmaf(a.z, wz[p], fmaf(a.y, wy[p], a.x * wx[p]));
        if (FR) {
            const float sp = db - lin;
            lin = fmaf(fmaf(-sp, sp, a.w), hq[p], lin);
        }
        const float r = mk_frac_nearest(lin);
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

template <int PIX, bool FR, bool CPLX>
__device__ __forceinline__ void mk_tile_terms(const float4 *__restrict__ P,
                                              const float4 *__restrict__ E, int T,
                                              const float (&wx)[PIX], const float (&wy)[PIX],
                                              const float (&wz)[PIX], const float (&hq)[PIX],
                                              float bx, float by, float bz, float (&csr)[PIX],
                                              float (&csi)[PIX])
{
#pragma unroll 2
    for (int q = 0; q < T / 2; ++q) {
        MkAtom u, v;
        mk_atom_pair(P, E, q, u, v);
        mk_atom_terms<PIX, FR, CPLX>(u, wx, wy, wz, hq, bx, by, bz, csr, csi);
        mk_atom_terms<PIX, FR, CPLX>(v, wx, wy, wz, hq, bx, by, bz, csr, csi);
    }
}

// The terms of one tile with a per-atom analyser multiplier
//   m = (t <= th) ? g0 + g1 t : 0,   t = D.g (the change of the squared chord
// |r_hat - c|^2 across the tile, linear in the offset D). Top-hat pixels that
// straddle the acceptance edge in this tile use (th = x_accept - x0, g0 = 1,
// g1 = 0); Darwin pixels the first-order expansion of the roll-off
// (th = inf); pixels with one factor for the whole tile (g0, g1 = 0, inf).
template <int PIX, bool FR, bool CPLX>
__device__ __forceinline__ void mk_atom_terms_ana(
    const MkAtom &at, const float (&wx)[PIX], const float (&wy)[PIX], const float (&wz)[PIX],
    const float (&hq)[PIX], float bx, float by, float bz, const float (&gx)[PIX],
    const float (&gy)[PIX], const float (&gz)[PIX], const float (&th)[PIX],
    const float (&g0)[PIX], const float (&g1)[PIX], float (&csr)[PIX], float (&csi)[PIX])
{
    const float4 a = at.a;
    const float2 e = at.e;
    float db = 0.f;
    if (FR) db = fmaf(a.z, bz, fmaf(a.y, by, a.x * bx));
#pragma unroll
    for (int p = 0; p < PIX; ++p) {
        float lin = fmaf(a.z, wz[p], fmaf(a.y, wy[p], a.x * wx[p]));
        if (FR) {
            const float sp = db - lin;
            lin = fmaf(fmaf(-sp, sp, a.w), hq[p], lin);
        }
        const float t = fmaf(a.z, gz[p], fmaf(a.y, gy[p], a.x * gx[p]));
        const float m = t <= th[p] ? fmaf(g1[p], t, g0[p]) : 0.f;
        const float r = mk_frac_nearest(lin);
        float sn, cs;
        __sincosf(r * TWO_PI_F, &sn, &cs);
        const float er = e.x * m;
        if (CPLX) {
            const float ei = e.y * m;
            csr[p] = fmaf(er, cs, fmaf(-ei, sn, csr[p]));
            csi[p] = fmaf(er, sn, fmaf(ei, cs, csi[p]));
        } else {
            csr[p] = fmaf(er, cs, csr[p]);
            csi[p] = fmaf(er, sn, csi[p]);
        }
    }
}

template <int PIX, bool FR, bool CPLX>
__device__ __forceinline__ void mk_tile_terms_ana(
    const float4 *__restrict__ P, const float4 *__restrict__ E, int T, const float (&wx)[PIX],
    const float (&wy)[PIX], const float (&wz)[PIX], const float (&hq)[PIX], float bx, float by,
    float bz, const float (&gx)[PIX], const float (&gy)[PIX], const float (&gz)[PIX],
    const float (&th)[PIX], const float (&g0)[PIX], const float (&g1)[PIX], float (&csr)[PIX],
    float (&csi)[PIX])
{
    for (int q = 0; q < T / 2; ++q) {
        MkAtom u, v;
        mk_atom_pair(P, E, q, u, v);
        mk_atom_terms_ana<PIX, FR, CPLX>(u, wx, wy, wz, hq, bx, by, bz, gx, gy, gz, th, g0, g1, csr, csi);
        mk_atom_terms_ana<PIX, FR, CPLX>(v, wx, wy, wz, hq, bx, by, bz, gx, gy, gz, th, g0, g1, csr, csi);
    }
}

// Packed FP32 pairs: f32x2 instructions (sm_100 and later) apply one IEEE
// fp32 operation to both halves of a 64-bit register pair. The pair loop
// below keeps two atoms in the two halves, so one instruction does the work
// of two (the FMA pipe's float rate is unchanged; issue slots halve).
typedef unsigned long long mk_f2;
__device__ __forceinline__ mk_f2 f2_pack(float lo, float hi)
{
    mk_f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ float2 f2_unpack(mk_f2 v)
{
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
    return r;
}
__device__ __forceinline__ mk_f2 f2_fma(mk_f2 a, mk_f2 b, mk_f2 c)
{
    mk_f2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ mk_f2 f2_mul(mk_f2 a, mk_f2 b)
{
    mk_f2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ mk_f2 f2_add(mk_f2 a, mk_f2 b)
{
    mk_f2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ mk_f2 f2_sub(mk_f2 a, mk_f2 b)
{
    mk_f2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ mk_f2 f2_splat(float x) { return f2_pack(x, x); }

// Pixel pairs (a, b) that are neighbours on the detector: with
// sigma = D.(w_a + w_b)/2 (cycles) and delta = pi D.(w_a - w_b) (radians),
//   exp(2 pi i D.w_a) = exp(2 pi i sigma) exp(+i delta),
//   exp(2 pi i D.w_b) = exp(2 pi i sigma) exp(-i delta).
// sigma takes the MUFU sin/cos; delta is small (|delta| <= pi |D| |w_a - w_b|,
// bounded by the host), so cos/sin(delta) are Taylor polynomials on the FMA
// pipe, with the atom's (real) amplitude e folded into their coefficients:
//   SHORT (|delta| <= MK_PAIR_SHORT_DELTA): e cos = e - (e/2) d^2,
//         e sin = delta (e - (e/6) d^2); truncation below delta^4/24 = 1e-6;
//   long  (|delta| <= 0.5): through d^6 and d^5; below delta^7/7! = 1.6e-6.
// One MUFU sin/cos for two terms instead of two. Sums kept as
// P = sum e e^{i sigma} cos(delta) and S = sum e e^{i sigma} sin(delta)
// (Q = i S); pixel a = P + i S, pixel b = P - i S. Every quantity of the
// loop is an f32x2 pair over the tile's atoms 2q and 2q+1 (interleaved in
// shared memory); the two halves of the accumulators are added at the end.
#define MK_PAIR_SHORT_DELTA 0.07f
// Default largest in-tile phase [rad] handed to the MUFU sin/cos without the
// mod-1 reduction (quad kernels; mk_launch.sin_direct_max_rad). __sincosf's absolute error grows about linearly
// with |x| (its argument scaling by 1/2pi rounds in FP32): measured on sm_103
// over uniform sweeps, at most 3.5e-7 in [-pi, pi], 1.0e-5 below 32 pi and
// 1.7e-5 just above. Below 100 rad the added error is of the size of the
// rounding of the FP32 in-tile phase itself, and like it differs from atom to
// atom.
#ifndef MK_SIN_DIRECT_MAX
#define MK_SIN_DIRECT_MAX 100.0f
#endif
#ifndef MK_PAIR_UNROLL
#define MK_PAIR_UNROLL 32
#endif
constexpr int kPairUnroll = MK_PAIR_UNROLL / 2;   // atom pairs per unrolled step
template <int NPAIR, bool FR, bool CPLX, bool SHORT>
__device__ __forceinline__ void mk_tile_terms_pair(
    const float4 *__restrict__ P, const float4 *__restrict__ E, int T, const mk_f2 (&sx)[NPAIR],
    const mk_f2 (&sy)[NPAIR], const mk_f2 (&sz)[NPAIR], const mk_f2 (&dx)[NPAIR],
    const mk_f2 (&dy)[NPAIR], const mk_f2 (&dz)[NPAIR], const mk_f2 (&hq)[NPAIR], mk_f2 bx,
    mk_f2 by, mk_f2 bz, mk_f2 (&pr)[NPAIR], mk_f2 (&pi)[NPAIR], mk_f2 (&sr)[NPAIR],
    mk_f2 (&si)[NPAIR])
{
    const mk_f2 magic = f2_splat(MK_ROUND_MAGIC), two_pi = f2_splat(TWO_PI_F);
    const mk_f2 one = f2_splat(1.f), m_one = f2_splat(-1.f);
    const mk_f2 k2 = f2_splat(-0.5f), k3 = f2_splat(-1.f / 6.f);
    const mk_f2 k4 = f2_splat(1.f / 24.f), k5 = f2_splat(1.f / 120.f), k6 = f2_splat(-1.f / 720.f);
    const ulonglong2 *P2 = reinterpret_cast<const ulonglong2 *>(P);
    const ulonglong2 *E2 = reinterpret_cast<const ulonglong2 *>(E);
#pragma unroll (kPairUnroll)
    for (int q = 0; q < T / 2; ++q) {
        const ulonglong2 A = P2[2 * q], B = P2[2 * q + 1], M = E2[q];
        const mk_f2 X = A.x, Y = A.y, Z = B.x, W = B.y, ER = M.x, EI = M.y;
        mk_f2 db = 0ull;
        if (FR) db = f2_fma(Z, bz, f2_fma(Y, by, f2_mul(X, bx)));
        // per-atom polynomial coefficients (amplitude folded in when real)
        const mk_f2 e0 = CPLX ? one : ER;
        const mk_f2 c2 = f2_mul(e0, k2), s2 = f2_mul(e0, k3);
        mk_f2 c4 = 0ull, s4 = 0ull, c6 = 0ull;
        if (!SHORT) {
            c4 = f2_mul(e0, k4);
            s4 = f2_mul(e0, k5);
            c6 = f2_mul(e0, k6);
        }
        mk_f2 EIn = 0ull;
        if (CPLX) EIn = f2_mul(EI, m_one);
#pragma unroll
        for (int p = 0; p < NPAIR; ++p) {
            mk_f2 sig = f2_fma(Z, sz[p], f2_fma(Y, sy[p], f2_mul(X, sx[p])));
            if (FR) {
                const mk_f2 sp = f2_sub(db, sig);
                sig = f2_fma(f2_fma(f2_mul(sp, m_one), sp, W), hq[p], sig);
            }
            const mk_f2 del = f2_fma(Z, dz[p], f2_fma(Y, dy[p], f2_mul(X, dx[p])));
            const mk_f2 rr = f2_mul(f2_sub(sig, f2_sub(f2_add(sig, magic), magic)), two_pi);
            const float2 r = f2_unpack(rr);
            float s0, c0, s1, c1;
            __sincosf(r.x, &s0, &c0);
            __sincosf(r.y, &s1, &c1);
            mk_f2 ec = f2_pack(c0, c1), es = f2_pack(s0, s1);
            const mk_f2 d2 = f2_mul(del, del);
            mk_f2 cd, sd;
            if (SHORT) {
                cd = f2_fma(d2, c2, e0);
                sd = f2_mul(del, f2_fma(d2, s2, e0));
            } else {
                cd = f2_fma(d2, f2_fma(d2, f2_fma(d2, c6, c4), c2), e0);
                sd = f2_mul(del, f2_fma(d2, f2_fma(d2, s4, s2), e0));
            }
            if (CPLX) {
                const mk_f2 c = ec;
                ec = f2_fma(ER, c, f2_mul(EIn, es));
                es = f2_fma(ER, es, f2_mul(EI, c));
            }
            pr[p] = f2_fma(ec, cd, pr[p]);
            pi[p] = f2_fma(es, cd, pi[p]);
            sr[p] = f2_fma(es, sd, sr[p]);
            si[p] = f2_fma(ec, sd, si[p]);
        }
    }
}

// 2x2 pixel quads: pixels a, b neighbours in one detector row, c, d the two
// below them. With sigma = D.(w_a + w_b + w_c + w_d)/4 (cycles),
// u = (pi/2) D.(w_b + w_d - w_a - w_c) (along the row, radians),
// v = (pi/2) D.(w_c + w_d - w_a - w_b) (across rows), and signs
// (s, t) = (-,-), (+,-), (-,+), (+,+) for a, b, c, d,
//   2 pi D.w = 2 pi sigma + s u + t v + s t x,
// x = (pi/2) D.(w_a + w_d - w_b - w_c) the mixed second difference, which is
// dropped (bounded by the host against its phase budget; it is of order
// k |D| (pixel / distance)^2). Then
//   e^{2 pi i D.w} = e^{2 pi i sigma} (cos u + i s sin u)(cos v + i t sin v)
//                  = e^{2 pi i sigma} [C_u C_v - s t S_u S_v + i (t C_u S_v + s S_u C_v)],
// one MUFU sin/cos for four terms; cos/sin of u and v are the pair
// polynomials (the atom's real amplitude folded into the u factor). The
// four sums K = sum E e^{2 pi i sigma} C_u C_v, R = ... C_u S_v,
// S = ... S_u C_v, Q = ... S_u S_v give every pixel of the quad:
//   A(s, t) = K - s t Q + i t R + i s S.
// acc[j][0..7] = K, R, S, Q (re, im) of quad j, f32x2 over atoms 2q, 2q+1.
// RAD (tiles without the |d|^2 term whose in-tile phase stays within
// MK_SIN_DIRECT_MAX radians): (sx, sy, sz) come scaled by 2 pi, so sigma is
// in radians and goes to the sin/cos without the mod-1 reduction.
template <int NQ, bool FR, bool CPLX, bool SHORT, bool RAD = false>
__device__ __forceinline__ void mk_tile_terms_quad(
    const float4 *__restrict__ P, const float4 *__restrict__ E, int T, const mk_f2 (&sx)[NQ],
    const mk_f2 (&sy)[NQ], const mk_f2 (&sz)[NQ], const mk_f2 (&ux)[NQ], const mk_f2 (&uy)[NQ],
    const mk_f2 (&uz)[NQ], const mk_f2 (&vx)[NQ], const mk_f2 (&vy)[NQ], const mk_f2 (&vz)[NQ],
    const mk_f2 (&hq)[NQ], mk_f2 bx, mk_f2 by, mk_f2 bz, mk_f2 (&acc)[NQ][8])
{
    const mk_f2 magic = f2_splat(MK_ROUND_MAGIC), two_pi = f2_splat(TWO_PI_F);
    const mk_f2 one = f2_splat(1.f), m_one = f2_splat(-1.f);
    const mk_f2 k2 = f2_splat(-0.5f), k3 = f2_splat(-1.f / 6.f);
    const mk_f2 k4 = f2_splat(1.f / 24.f), k5 = f2_splat(1.f / 120.f), k6 = f2_splat(-1.f / 720.f);
    const ulonglong2 *P2 = reinterpret_cast<const ulonglong2 *>(P);
    const ulonglong2 *E2 = reinterpret_cast<const ulonglong2 *>(E);
#pragma unroll (kPairUnroll)
    for (int q = 0; q < T / 2; ++q) {
        const ulonglong2 A = P2[2 * q], B = P2[2 * q + 1], M = E2[q];
        const mk_f2 X = A.x, Y = A.y, Z = B.x, W = B.y, ER = M.x, EI = M.y;
        mk_f2 db = 0ull;
        if (FR) db = f2_fma(Z, bz, f2_fma(Y, by, f2_mul(X, bx)));
        const mk_f2 e0 = CPLX ? one : ER;
        const mk_f2 c2 = f2_mul(e0, k2), s2 = f2_mul(e0, k3);
        mk_f2 c4 = 0ull, s4 = 0ull, c6 = 0ull;
        if (!SHORT) {
            c4 = f2_mul(e0, k4);
            s4 = f2_mul(e0, k5);
            c6 = f2_mul(e0, k6);
        }
        mk_f2 EIn = 0ull;
        if (CPLX) EIn = f2_mul(EI, m_one);
#pragma unroll
        for (int j = 0; j < NQ; ++j) {
            mk_f2 sig = f2_fma(Z, sz[j], f2_fma(Y, sy[j], f2_mul(X, sx[j])));
            if (FR) {
                const mk_f2 sp = f2_sub(db, sig);
                sig = f2_fma(f2_fma(f2_mul(sp, m_one), sp, W), hq[j], sig);
            }
            const mk_f2 du = f2_fma(Z, uz[j], f2_fma(Y, uy[j], f2_mul(X, ux[j])));
            const mk_f2 dv = f2_fma(Z, vz[j], f2_fma(Y, vy[j], f2_mul(X, vx[j])));
            const mk_f2 rr = RAD ? sig : f2_mul(f2_sub(sig, f2_sub(f2_add(sig, magic), magic)), two_pi);
            const float2 r = f2_unpack(rr);
            float s0, c0, s1, c1;
            __sincosf(r.x, &s0, &c0);
            __sincosf(r.y, &s1, &c1);
            mk_f2 ec = f2_pack(c0, c1), es = f2_pack(s0, s1);
            if (CPLX) {
                const mk_f2 c = ec;
                ec = f2_fma(ER, c, f2_mul(EIn, es));
                es = f2_fma(ER, es, f2_mul(EI, c));
            }
            const mk_f2 u2 = f2_mul(du, du), v2 = f2_mul(dv, dv);
            mk_f2 cu, su, cv, sv;
            if (SHORT) {
                cu = f2_fma(u2, c2, e0);
                su = f2_mul(du, f2_fma(u2, s2, e0));
                cv = f2_fma(v2, k2, one);
                sv = f2_mul(dv, f2_fma(v2, k3, one));
            } else {
                cu = f2_fma(u2, f2_fma(u2, f2_fma(u2, c6, c4), c2), e0);
                su = f2_mul(du, f2_fma(u2, f2_fma(u2, s4, s2), e0));
                cv = f2_fma(v2, f2_fma(v2, f2_fma(v2, k6, k4), k2), one);
                sv = f2_mul(dv, f2_fma(v2, f2_fma(v2, k5, k3), one));
            }
            const mk_f2 xc = f2_mul(ec, cu), yc = f2_mul(es, cu);
            const mk_f2 xs = f2_mul(ec, su), ys = f2_mul(es, su);
            acc[j][0] = f2_fma(xc, cv, acc[j][0]);
            acc[j][1] = f2_fma(yc, cv, acc[j][1]);
            acc[j][2] = f2_fma(xc, sv, acc[j][2]);
            acc[j][3] = f2_fma(yc, sv, acc[j][3]);
            acc[j][4] = f2_fma(xs, cv, acc[j][4]);
            acc[j][5] = f2_fma(ys, cv, acc[j][5]);
            acc[j][6] = f2_fma(xs, sv, acc[j][6]);
            acc[j][7] = f2_fma(ys, sv, acc[j][7]);
        }
    }
}

// 2x4 pixel octets: two 2x2 quads side by side in a pair of detector rows
// (a b a' b' in the upper row, c d c' d' below) share one pair of half
// differences u, v -- the means of the two quads' -- and take their quad
// phases from the octet's mean phase sigma_c: the quad centres sit one pixel
// step either side of the octet centre, and a pixel step is 2u, so
//   2 pi sigma_0 = 2 pi sigma_c - 2 u,   2 pi sigma_1 = 2 pi sigma_c + 2 u,
// and inside quad j the quad form applies unchanged. Dropped beyond the quad
// form: the change of the row and column steps across the octet (the
// octet's departure from a plane in w), which the host bounds from the
// FP64 pixel directions against its phase budget. Per atom pair: three dot
// products (9), the two quad phases (2), two sin/cos, u^2 and v^2 (2), the
// polynomials (6), 2 x 4 products with the phasors and 2 x 8 accumulators:
// ~45 FP32 lane operations per 8 terms (two quads: ~60).
// acc[j][0..7] = K, R, S, Q (re, im) of quad j, f32x2 over atoms 2q, 2q+1.
template <bool FR, bool CPLX, bool SHORT, bool RAD>
__device__ __forceinline__ void mk_tile_terms_oct(
    const float4 *__restrict__ P, const float4 *__restrict__ E, int T, mk_f2 sx, mk_f2 sy, mk_f2 sz,
    mk_f2 ux, mk_f2 uy, mk_f2 uz, mk_f2 vx, mk_f2 vy, mk_f2 vz, mk_f2 hq, mk_f2 bx, mk_f2 by,
    mk_f2 bz, mk_f2 (&acc)[2][8])
{
    const mk_f2 magic = f2_splat(MK_ROUND_MAGIC), two_pi = f2_splat(TWO_PI_F);
    const mk_f2 one = f2_splat(1.f), m_one = f2_splat(-1.f);
    const mk_f2 two = f2_splat(2.f), m_two = f2_splat(-2.f);
    const mk_f2 k2 = f2_splat(-0.5f), k3 = f2_splat(-1.f / 6.f);
    const mk_f2 k4 = f2_splat(1.f / 24.f), k5 = f2_splat(1.f / 120.f), k6 = f2_splat(-1.f / 720.f);
    const ulonglong2 *P2 = reinterpret_cast<const ulonglong2 *>(P);
    const ulonglong2 *E2 = reinterpret_cast<const ulonglong2 *>(E);
#pragma unroll (kPairUnroll)
    for (int q = 0; q < T / 2; ++q) {
        const ulonglong2 A = P2[2 * q], B = P2[2 * q + 1], M = E2[q];
        const mk_f2 X = A.x, Y = A.y, Z = B.x, W = B.y, ER = M.x, EI = M.y;
        const mk_f2 e0 = CPLX ? one : ER;
        const mk_f2 c2 = f2_mul(e0, k2), s2 = f2_mul(e0, k3);
        mk_f2 c4 = 0ull, s4 = 0ull, c6 = 0ull;
        if (!SHORT) {
            c4 = f2_mul(e0, k4);
            s4 = f2_mul(e0, k5);
            c6 = f2_mul(e0, k6);
        }
        mk_f2 sig = f2_fma(Z, sz, f2_fma(Y, sy, f2_mul(X, sx)));
        if (FR) {
            const mk_f2 db = f2_fma(Z, bz, f2_fma(Y, by, f2_mul(X, bx)));
            const mk_f2 sp = f2_sub(db, sig);
            sig = f2_fma(f2_fma(f2_mul(sp, m_one), sp, W), hq, sig);
        }
        const mk_f2 du = f2_fma(Z, uz, f2_fma(Y, uy, f2_mul(X, ux)));
        const mk_f2 dv = f2_fma(Z, vz, f2_fma(Y, vy, f2_mul(X, vx)));
        const mk_f2 rc = RAD ? sig : f2_mul(f2_sub(sig, f2_sub(f2_add(sig, magic), magic)), two_pi);
        const float2 r0 = f2_unpack(f2_fma(du, m_two, rc));
        const float2 r1 = f2_unpack(f2_fma(du, two, rc));
        float sa, ca, sb, cb, sc_, cc, sd, cd;
        __sincosf(r0.x, &sa, &ca);
        __sincosf(r0.y, &sb, &cb);
        __sincosf(r1.x, &sc_, &cc);
        __sincosf(r1.y, &sd, &cd);
        mk_f2 ec[2] = {f2_pack(ca, cb), f2_pack(cc, cd)};
        mk_f2 es[2] = {f2_pack(sa, sb), f2_pack(sc_, sd)};
        if (CPLX) {
            const mk_f2 EIn = f2_mul(EI, m_one);
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const mk_f2 c = ec[j];
                ec[j] = f2_fma(ER, c, f2_mul(EIn, es[j]));
                es[j] = f2_fma(ER, es[j], f2_mul(EI, c));
            }
        }
        const mk_f2 u2 = f2_mul(du, du), v2 = f2_mul(dv, dv);
        mk_f2 cu, su, cv, sv;
        if (SHORT) {
            cu = f2_fma(u2, c2, e0);
            su = f2_mul(du, f2_fma(u2, s2, e0));
            cv = f2_fma(v2, k2, one);
            sv = f2_mul(dv, f2_fma(v2, k3, one));
        } else {
            cu = f2_fma(u2, f2_fma(u2, f2_fma(u2, c6, c4), c2), e0);
            su = f2_mul(du, f2_fma(u2, f2_fma(u2, s4, s2), e0));
            cv = f2_fma(v2, f2_fma(v2, f2_fma(v2, k6, k4), k2), one);
            sv = f2_mul(dv, f2_fma(v2, f2_fma(v2, k5, k3), one));
        }
        // the two quads share u and v: the four products of their factors
        // are formed once and each quad's 8 sums take one FMA apiece
        const mk_f2 pcc = f2_mul(cu, cv), pcs = f2_mul(cu, sv);
        const mk_f2 psc = f2_mul(su, cv), pss = f2_mul(su, sv);
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            acc[j][0] = f2_fma(ec[j], pcc, acc[j][0]);
            acc[j][1] = f2_fma(es[j], pcc, acc[j][1]);
            acc[j][2] = f2_fma(ec[j], pcs, acc[j][2]);
            acc[j][3] = f2_fma(es[j], pcs, acc[j][3]);
            acc[j][4] = f2_fma(ec[j], psc, acc[j][4]);
            acc[j][5] = f2_fma(es[j], psc, acc[j][5]);
            acc[j][6] = f2_fma(ec[j], pss, acc[j][6]);
            acc[j][7] = f2_fma(es[j], pss, acc[j][7]);
        }
    }
}

// 4x4 pixel squares: four 2x2 quads in a 2x2 arrangement (quad j at row
// pair j >> 1 and column pair j & 1 of the square) share one pair of half
// differences u, v -- the means of the four quads' -- and take their quad
// phases from the square's mean phase sigma_c: each quad centre sits one
// pixel step from the square centre along the row and one across it, a row
// step is 2u and a column step 2v, so
//   2 pi sigma_j = 2 pi sigma_c + s_j 2u + t_j 2v,   s_j = +-1, t_j = +-1,
// and inside quad j the quad form applies unchanged. Dropped beyond the
// quad form: the departure of w over the 16 pixels from a plane, which the
// host bounds from the FP64 pixel directions against its phase budget. Per
// atom: three dot products (9), the four quad phases (6), the four sin/cos
// argument scalings (4), u^2 and v^2 (2), the polynomials (6), the four
// products of the shared factors (4), 4 x 8 accumulators (32) and the
// amplitude coefficients (2): 65 FP32 lane operations for 16 terms on tiles
// that pass the phase straight to the sin/cos (4.1 a term, against 5.4 for
// octets), with the MUFU doing one sin/cos per 4 terms as in every quad form.
// acc[j][0..7] = K, R, S, Q (re, im) of quad j, f32x2 over atoms 2q, 2q+1.
// Unrolled by 8 atom pairs, not 16 as the other forms: held to ~168
// registers, the square loop ran the 8.19M-atom exposure 3.9 % faster so.
#ifndef MK_SQ_PAIR_UNROLL
#define MK_SQ_PAIR_UNROLL 8
#endif
constexpr int kSqPairUnroll = MK_SQ_PAIR_UNROLL;
template <bool FR, bool CPLX, bool SHORT, bool RAD>
__device__ __forceinline__ void mk_tile_terms_sq(
    const float4 *__restrict__ P, const float4 *__restrict__ E, int T, mk_f2 sx, mk_f2 sy, mk_f2 sz,
    mk_f2 ux, mk_f2 uy, mk_f2 uz, mk_f2 vx, mk_f2 vy, mk_f2 vz, mk_f2 hq, mk_f2 bx, mk_f2 by,
    mk_f2 bz, mk_f2 (&acc)[4][8])
{
    const mk_f2 magic = f2_splat(MK_ROUND_MAGIC), two_pi = f2_splat(TWO_PI_F);
    const mk_f2 one = f2_splat(1.f), m_one = f2_splat(-1.f);
    const mk_f2 two = f2_splat(2.f), m_two = f2_splat(-2.f);
    const mk_f2 k2 = f2_splat(-0.5f), k3 = f2_splat(-1.f / 6.f);
    const mk_f2 k4 = f2_splat(1.f / 24.f), k5 = f2_splat(1.f / 120.f), k6 = f2_splat(-1.f / 720.f);
    const ulonglong2 *P2 = reinterpret_cast<const ulonglong2 *>(P);
    const ulonglong2 *E2 = reinterpret_cast<const ulonglong2 *>(E);
#pragma unroll (kSqPairUnroll)
    for (int q = 0; q < T / 2; ++q) {
        const ulonglong2 A = P2[2 * q], B = P2[2 * q + 1], M = E2[q];
        const mk_f2 X = A.x, Y = A.y, Z = B.x, W = B.y, ER = M.x, EI = M.y;
        const mk_f2 e0 = CPLX ? one : ER;
        const mk_f2 c2 = f2_mul(e0, k2), s2 = f2_mul(e0, k3);
        mk_f2 c4 = 0ull, s4 = 0ull, c6 = 0ull;
        if (!SHORT) {
            c4 = f2_mul(e0, k4);
            s4 = f2_mul(e0, k5);
            c6 = f2_mul(e0, k6);
        }
        mk_f2 sig = f2_fma(Z, sz, f2_fma(Y, sy, f2_mul(X, sx)));
        if (FR) {
            const mk_f2 db = f2_fma(Z, bz, f2_fma(Y, by, f2_mul(X, bx)));
            const mk_f2 sp = f2_sub(db, sig);
            sig = f2_fma(f2_fma(f2_mul(sp, m_one), sp, W), hq, sig);
        }
        const mk_f2 du = f2_fma(Z, uz, f2_fma(Y, uy, f2_mul(X, ux)));
        const mk_f2 dv = f2_fma(Z, vz, f2_fma(Y, vy, f2_mul(X, vx)));
        const mk_f2 rc = RAD ? sig : f2_mul(f2_sub(sig, f2_sub(f2_add(sig, magic), magic)), two_pi);
        // quad phases: rows t = -1 (quads 0, 1) and t = +1 (quads 2, 3),
        // columns s = -1 (quads 0, 2) and s = +1 (quads 1, 3)
        const mk_f2 rlo = f2_fma(dv, m_two, rc), rhi = f2_fma(dv, two, rc);
        const float2 r0 = f2_unpack(f2_fma(du, m_two, rlo));
        const float2 r1 = f2_unpack(f2_fma(du, two, rlo));
        const float2 r2 = f2_unpack(f2_fma(du, m_two, rhi));
        const float2 r3 = f2_unpack(f2_fma(du, two, rhi));
        mk_f2 ec[4], es[4];
        {
            float s0, c0, s1, c1;
            __sincosf(r0.x, &s0, &c0);
            __sincosf(r0.y, &s1, &c1);
            ec[0] = f2_pack(c0, c1); es[0] = f2_pack(s0, s1);
            __sincosf(r1.x, &s0, &c0);
            __sincosf(r1.y, &s1, &c1);
            ec[1] = f2_pack(c0, c1); es[1] = f2_pack(s0, s1);
            __sincosf(r2.x, &s0, &c0);
            __sincosf(r2.y, &s1, &c1);
            ec[2] = f2_pack(c0, c1); es[2] = f2_pack(s0, s1);
            __sincosf(r3.x, &s0, &c0);
            __sincosf(r3.y, &s1, &c1);
            ec[3] = f2_pack(c0, c1); es[3] = f2_pack(s0, s1);
        }
        if (CPLX) {
            const mk_f2 EIn = f2_mul(EI, m_one);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const mk_f2 c = ec[j];
                ec[j] = f2_fma(ER, c, f2_mul(EIn, es[j]));
                es[j] = f2_fma(ER, es[j], f2_mul(EI, c));
            }
        }
        const mk_f2 u2 = f2_mul(du, du), v2 = f2_mul(dv, dv);
        mk_f2 cu, su, cv, sv;
        if (SHORT) {
            cu = f2_fma(u2, c2, e0);
            su = f2_mul(du, f2_fma(u2, s2, e0));
            cv = f2_fma(v2, k2, one);
            sv = f2_mul(dv, f2_fma(v2, k3, one));
        } else {
            cu = f2_fma(u2, f2_fma(u2, f2_fma(u2, c6, c4), c2), e0);
            su = f2_mul(du, f2_fma(u2, f2_fma(u2, s4, s2), e0));
            cv = f2_fma(v2, f2_fma(v2, f2_fma(v2, k6, k4), k2), one);
            sv = f2_mul(dv, f2_fma(v2, f2_fma(v2, k5, k3), one));
        }
        const mk_f2 pcc = f2_mul(cu, cv), pcs = f2_mul(cu, sv);
        const mk_f2 psc = f2_mul(su, cv), pss = f2_mul(su, sv);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            acc[j][0] = f2_fma(ec[j], pcc, acc[j][0]);
            acc[j][1] = f2_fma(es[j], pcc, acc[j][1]);
            acc[j][2] = f2_fma(ec[j], pcs, acc[j][2]);
            acc[j][3] = f2_fma(es[j], pcs, acc[j][3]);
            acc[j][4] = f2_fma(ec[j], psc, acc[j][4]);
            acc[j][5] = f2_fma(es[j], psc, acc[j][5]);
            acc[j][6] = f2_fma(ec[j], pss, acc[j][6]);
            acc[j][7] = f2_fma(es[j], pss, acc[j][7]);
        }
    }
}

// PM (pixel mode): 0 one sin/cos a term, 1 pixel pairs, 2 pixel quads, 3
// pixel octets (2x4: two quads sharing their half differences), 4 pixel
// squares (4x4: four quads sharing them).
// Blocks per SM the register allocation is held to: the 8-pixel quad kernels
// (their per-pixel state lives in shared memory) aim at MK_QUAD8_WARPS warps
// per SM, the rest are free.
#ifndef MK_QUAD8_WARPS
#define MK_QUAD8_WARPS 12
#endif
#ifndef MK_OCT_WARPS
#define MK_OCT_WARPS 12
#endif
#ifndef MK_SQ_WARPS
#define MK_SQ_WARPS 12
#endif
template <int NT, int PIX, int PM, bool ANA>
constexpr int mk_min_blocks()
{
    return (PM == 2 && PIX == 8 && !ANA && MK_QUAD8_WARPS * 32 / NT > 1) ? MK_QUAD8_WARPS * 32 / NT
           : (PM == 3 && MK_OCT_WARPS * 32 / NT > 1)                  ? MK_OCT_WARPS * 32 / NT
           : (PM == 4 && MK_SQ_WARPS * 32 / NT > 1)                   ? MK_SQ_WARPS * 32 / NT
                                                                       : 1;
}

// The 2x2 pixel-quad form for one tile: NQ quads of the thread (pixels
// 4j..4j+3 = a, b, c, d), each with its own mean, half differences and
// sin/cos; the quad kernels run it on every tile and the octet kernels on
// tiles too wide for the octet form.
template <int NQ, bool CPLX>
__device__ __forceinline__ void mk_quads_tile(const MkSplitArgs &A, const mk_frame_desc &F,
                                              const double4 &o, bool fr_tile,
                                              const float4 *__restrict__ P,
                                              const float4 *__restrict__ E, int T,
                                              const float (&wx)[4 * NQ], const float (&wy)[4 * NQ],
                                              const float (&wz)[4 * NQ], const float (&hq)[4 * NQ],
                                              float (&csr)[4 * NQ], float (&csi)[4 * NQ])
{
    mk_f2 sx[NQ], sy[NQ], sz[NQ], ux[NQ], uy[NQ], uz[NQ], vx[NQ], vy[NQ], vz[NQ],
        hp[NQ];
    mk_f2 acc[NQ][8];
#pragma unroll
    for (int j = 0; j < NQ; ++j) {
        const int a = 4 * j, b = a + 1, c = a + 2, d = a + 3;
        const float hpi = 1.57079632679490f;
        sx[j] = f2_splat(0.25f * ((wx[a] + wx[b]) + (wx[c] + wx[d])));
        sy[j] = f2_splat(0.25f * ((wy[a] + wy[b]) + (wy[c] + wy[d])));
        sz[j] = f2_splat(0.25f * ((wz[a] + wz[b]) + (wz[c] + wz[d])));
        ux[j] = f2_splat(hpi * ((wx[b] - wx[a]) + (wx[d] - wx[c])));
        uy[j] = f2_splat(hpi * ((wy[b] - wy[a]) + (wy[d] - wy[c])));
        uz[j] = f2_splat(hpi * ((wz[b] - wz[a]) + (wz[d] - wz[c])));
        vx[j] = f2_splat(hpi * ((wx[c] - wx[a]) + (wx[d] - wx[b])));
        vy[j] = f2_splat(hpi * ((wy[c] - wy[a]) + (wy[d] - wy[b])));
        vz[j] = f2_splat(hpi * ((wz[c] - wz[a]) + (wz[d] - wz[b])));
        hp[j] = f2_splat(0.25f * ((hq[a] + hq[b]) + (hq[c] + hq[d])));
#pragma unroll
        for (int m = 0; m < 8; ++m) acc[j][m] = 0ull;
    }
    const mk_f2 bx = f2_splat(F.b[0]), by = f2_splat(F.b[1]), bz = f2_splat(F.b[2]);
    const bool short_tile = (float)o.w <= A.pair_short_r;
    // direct sin/cos argument: warp-uniform, from the bound
    // 2 pi |w_mean| kappa r of every quad of the warp
    bool rad = false;
    if (!fr_tile && short_tile) {
        float wmax = 0.f;
#pragma unroll
        for (int j = 0; j < NQ; ++j) {
            const float2 a = f2_unpack(sx[j]), b = f2_unpack(sy[j]), c = f2_unpack(sz[j]);
            wmax = fmaxf(wmax, fmaf(c.x, c.x, fmaf(b.x, b.x, a.x * a.x)));
        }
        const float bound = TWO_PI_F * sqrtf(wmax) * A.kappa * (float)o.w;
        rad = __all_sync(0xffffffffu, bound <= A.sin_direct);
    }
    if (rad) {
#pragma unroll
        for (int j = 0; j < NQ; ++j) {
            sx[j] = f2_mul(sx[j], f2_splat(TWO_PI_F));
            sy[j] = f2_mul(sy[j], f2_splat(TWO_PI_F));
            sz[j] = f2_mul(sz[j], f2_splat(TWO_PI_F));
        }
        mk_tile_terms_quad<NQ, false, CPLX, true, true>(P, E, T, sx, sy, sz, ux, uy, uz,
                                                        vx, vy, vz, hp, bx, by, bz, acc);
    } else if (fr_tile) {
        if (short_tile)
            mk_tile_terms_quad<NQ, true, CPLX, true>(P, E, T, sx, sy, sz, ux, uy, uz, vx,
                                                     vy, vz, hp, bx, by, bz, acc);
        else
            mk_tile_terms_quad<NQ, true, CPLX, false>(P, E, T, sx, sy, sz, ux, uy, uz,
                                                      vx, vy, vz, hp, bx, by, bz, acc);
    } else {
        if (short_tile)
            mk_tile_terms_quad<NQ, false, CPLX, true>(P, E, T, sx, sy, sz, ux, uy, uz,
                                                      vx, vy, vz, hp, bx, by, bz, acc);
        else
            mk_tile_terms_quad<NQ, false, CPLX, false>(P, E, T, sx, sy, sz, ux, uy, uz,
                                                       vx, vy, vz, hp, bx, by, bz, acc);
    }
#pragma unroll
    for (int j = 0; j < NQ; ++j) {
        float h[8];
#pragma unroll
        for (int m = 0; m < 8; ++m) {
            const float2 t2 = f2_unpack(acc[j][m]);   // halves: even, odd atoms
            h[m] = t2.x + t2.y;
        }
        const float Kr = h[0], Ki = h[1], Rr = h[2], Ri = h[3];
        const float Sr = h[4], Si = h[5], Qr = h[6], Qi = h[7];
        // A(s, t) = K - s t Q + i t R + i s S
        csr[4 * j] = (Kr - Qr) + (Ri + Si);       // a (-, -)
        csi[4 * j] = (Ki - Qi) - (Rr + Sr);
        csr[4 * j + 1] = (Kr + Qr) + (Ri - Si);   // b (+, -)
        csi[4 * j + 1] = (Ki + Qi) - (Rr - Sr);
        csr[4 * j + 2] = (Kr + Qr) - (Ri - Si);   // c (-, +)
        csi[4 * j + 2] = (Ki + Qi) + (Rr - Sr);
        csr[4 * j + 3] = (Kr - Qr) - (Ri + Si);   // d (+, +)
        csi[4 * j + 3] = (Ki - Qi) + (Rr + Sr);
    }
}

// The 2x4 pixel-octet form for one tile (pixels 0..3 and 4..7 are the
// thread's two quads a, b, c, d, side by side).
template <bool CPLX>
__device__ __forceinline__ void mk_octet_tile(const MkSplitArgs &A, const mk_frame_desc &F,
                                              const double4 &o, bool fr_tile,
                                              const float4 *__restrict__ P,
                                              const float4 *__restrict__ E, int T,
                                              const float (&wx)[8], const float (&wy)[8],
                                              const float (&wz)[8], const float (&hq)[8],
                                              float (&csr)[8], float (&csi)[8])
{
    // octet vectors: mean w of the 8 pixels, and the two quads'
    // mean half-difference vectors (pixels 0..3 and 4..7 are
    // quads a b c d)
    const float hpi4 = 0.785398163397448f;   // (pi/2) / 2 quads
    float msx = 0.f, msy = 0.f, msz = 0.f, mh = 0.f;
#pragma unroll
    for (int p = 0; p < 8; ++p) {
        msx += wx[p]; msy += wy[p]; msz += wz[p]; mh += hq[p];
    }
    const float ax = hpi4 * (((wx[1] - wx[0]) + (wx[3] - wx[2])) + ((wx[5] - wx[4]) + (wx[7] - wx[6])));
    const float ay = hpi4 * (((wy[1] - wy[0]) + (wy[3] - wy[2])) + ((wy[5] - wy[4]) + (wy[7] - wy[6])));
    const float az = hpi4 * (((wz[1] - wz[0]) + (wz[3] - wz[2])) + ((wz[5] - wz[4]) + (wz[7] - wz[6])));
    const float cx = hpi4 * (((wx[2] - wx[0]) + (wx[3] - wx[1])) + ((wx[6] - wx[4]) + (wx[7] - wx[5])));
    const float cy = hpi4 * (((wy[2] - wy[0]) + (wy[3] - wy[1])) + ((wy[6] - wy[4]) + (wy[7] - wy[5])));
    const float cz = hpi4 * (((wz[2] - wz[0]) + (wz[3] - wz[1])) + ((wz[6] - wz[4]) + (wz[7] - wz[5])));
    msx *= 0.125f; msy *= 0.125f; msz *= 0.125f; mh *= 0.125f;
    mk_f2 acc[2][8];
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int m = 0; m < 8; ++m) acc[j][m] = 0ull;
    const mk_f2 bx = f2_splat(F.b[0]), by = f2_splat(F.b[1]), bz = f2_splat(F.b[2]);
    const bool short_tile = (float)o.w <= A.pair_short_r;
    // direct sin/cos argument (warp-uniform): the quad phases
    // reach kappa r (2 pi |s| + 2 |u|)
    bool rad = false;
    if (!fr_tile && short_tile) {
        const float bound = (TWO_PI_F * sqrtf(fmaf(msz, msz, fmaf(msy, msy, msx * msx))) +
                             2.f * sqrtf(fmaf(az, az, fmaf(ay, ay, ax * ax)))) *
                            A.kappa * (float)o.w;
        rad = __all_sync(0xffffffffu, bound <= A.sin_direct);
    }
    const mk_f2 ux = f2_splat(ax), uy = f2_splat(ay), uz = f2_splat(az);
    const mk_f2 vx = f2_splat(cx), vy = f2_splat(cy), vz = f2_splat(cz);
    const mk_f2 hp = f2_splat(mh);
    if (rad) {
        const mk_f2 sx = f2_splat(msx * TWO_PI_F), sy = f2_splat(msy * TWO_PI_F),
                    sz = f2_splat(msz * TWO_PI_F);
        mk_tile_terms_oct<false, CPLX, true, true>(P, E, T, sx, sy, sz, ux, uy, uz, vx, vy,
                                                   vz, hp, bx, by, bz, acc);
    } else {
        const mk_f2 sx = f2_splat(msx), sy = f2_splat(msy), sz = f2_splat(msz);
        if (fr_tile) {
            if (short_tile)
                mk_tile_terms_oct<true, CPLX, true, false>(P, E, T, sx, sy, sz, ux, uy, uz,
                                                           vx, vy, vz, hp, bx, by, bz, acc);
            else
                mk_tile_terms_oct<true, CPLX, false, false>(P, E, T, sx, sy, sz, ux, uy,
                                                            uz, vx, vy, vz, hp, bx, by, bz,
                                                            acc);
        } else {
            if (short_tile)
                mk_tile_terms_oct<false, CPLX, true, false>(P, E, T, sx, sy, sz, ux, uy,
                                                            uz, vx, vy, vz, hp, bx, by, bz,
                                                            acc);
            else
                mk_tile_terms_oct<false, CPLX, false, false>(P, E, T, sx, sy, sz, ux, uy,
                                                             uz, vx, vy, vz, hp, bx, by,
                                                             bz, acc);
        }
    }
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        float h[8];
#pragma unroll
        for (int m = 0; m < 8; ++m) {
            const float2 t2 = f2_unpack(acc[j][m]);   // halves: even, odd atoms
            h[m] = t2.x + t2.y;
        }
        const float Kr = h[0], Ki = h[1], Rr = h[2], Ri = h[3];
        const float Sr = h[4], Si = h[5], Qr = h[6], Qi = h[7];
        // A(s, t) = K - s t Q + i t R + i s S
        csr[4 * j] = (Kr - Qr) + (Ri + Si);       // a (-, -)
        csi[4 * j] = (Ki - Qi) - (Rr + Sr);
        csr[4 * j + 1] = (Kr + Qr) + (Ri - Si);   // b (+, -)
        csi[4 * j + 1] = (Ki + Qi) - (Rr - Sr);
        csr[4 * j + 2] = (Kr + Qr) - (Ri - Si);   // c (-, +)
        csi[4 * j + 2] = (Ki + Qi) + (Rr - Sr);
        csr[4 * j + 3] = (Kr - Qr) - (Ri + Si);   // d (+, +)
        csi[4 * j + 3] = (Ki - Qi) + (Rr + Sr);
    }
}

// The 4x4 pixel-square form for one tile (pixels 4j..4j+3 are the thread's
// quad j = a, b, c, d at row pair j >> 1 and column pair j & 1).
template <bool CPLX>
__device__ __forceinline__ void mk_square_tile(const MkSplitArgs &A, const mk_frame_desc &F,
                                               const double4 &o, bool fr_tile,
                                               const float4 *__restrict__ P,
                                               const float4 *__restrict__ E, int T,
                                               const float (&wx)[16], const float (&wy)[16],
                                               const float (&wz)[16], const float (&hq)[16],
                                               float (&csr)[16], float (&csi)[16])
{
    // square vectors: mean w of the 16 pixels, and the four quads' mean
    // half-difference vectors along the row (u) and across rows (v)
    const float hpi4 = 0.392699081698724f;   // (pi/2) / 4 quads
    float msx = 0.f, msy = 0.f, msz = 0.f, mh = 0.f;
    float ax = 0.f, ay = 0.f, az = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
#pragma unroll
    for (int p = 0; p < 16; ++p) {
        msx += wx[p]; msy += wy[p]; msz += wz[p]; mh += hq[p];
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int a = 4 * j, b = a + 1, c = a + 2, d = a + 3;
        ax += (wx[b] - wx[a]) + (wx[d] - wx[c]);
        ay += (wy[b] - wy[a]) + (wy[d] - wy[c]);
        az += (wz[b] - wz[a]) + (wz[d] - wz[c]);
        cx += (wx[c] - wx[a]) + (wx[d] - wx[b]);
        cy += (wy[c] - wy[a]) + (wy[d] - wy[b]);
        cz += (wz[c] - wz[a]) + (wz[d] - wz[b]);
    }
    ax *= hpi4; ay *= hpi4; az *= hpi4; cx *= hpi4; cy *= hpi4; cz *= hpi4;
    msx *= 0.0625f; msy *= 0.0625f; msz *= 0.0625f; mh *= 0.0625f;
    mk_f2 acc[4][8];
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int m = 0; m < 8; ++m) acc[j][m] = 0ull;
    const mk_f2 bx = f2_splat(F.b[0]), by = f2_splat(F.b[1]), bz = f2_splat(F.b[2]);
    const bool short_tile = (float)o.w <= A.pair_short_r;
    // direct sin/cos argument (warp-uniform): the quad phases reach
    // kappa r (2 pi |s| + 2 |u| + 2 |v|)
    bool rad = false;
    if (!fr_tile && short_tile) {
        const float bound = (TWO_PI_F * sqrtf(fmaf(msz, msz, fmaf(msy, msy, msx * msx))) +
                             2.f * sqrtf(fmaf(az, az, fmaf(ay, ay, ax * ax))) +
                             2.f * sqrtf(fmaf(cz, cz, fmaf(cy, cy, cx * cx)))) *
                            A.kappa * (float)o.w;
        rad = __all_sync(0xffffffffu, bound <= A.sin_direct);
    }
    const mk_f2 ux = f2_splat(ax), uy = f2_splat(ay), uz = f2_splat(az);
    const mk_f2 vx = f2_splat(cx), vy = f2_splat(cy), vz = f2_splat(cz);
    const mk_f2 hp = f2_splat(mh);
    if (rad) {
        const mk_f2 sx = f2_splat(msx * TWO_PI_F), sy = f2_splat(msy * TWO_PI_F),
                    sz = f2_splat(msz * TWO_PI_F);
        mk_tile_terms_sq<false, CPLX, true, true>(P, E, T, sx, sy, sz, ux, uy, uz, vx, vy, vz,
                                                  hp, bx, by, bz, acc);
    } else {
        const mk_f2 sx = f2_splat(msx), sy = f2_splat(msy), sz = f2_splat(msz);
        if (fr_tile) {
            if (short_tile)
                mk_tile_terms_sq<true, CPLX, true, false>(P, E, T, sx, sy, sz, ux, uy, uz, vx,
                                                          vy, vz, hp, bx, by, bz, acc);
            else
                mk_tile_terms_sq<true, CPLX, false, false>(P, E, T, sx, sy, sz, ux, uy, uz, vx,
                                                           vy, vz, hp, bx, by, bz, acc);
        } else {
            if (short_tile)
                mk_tile_terms_sq<false, CPLX, true, false>(P, E, T, sx, sy, sz, ux, uy, uz, vx,
                                                           vy, vz, hp, bx, by, bz, acc);
            else
                mk_tile_terms_sq<false, CPLX, false, false>(P, E, T, sx, sy, sz, ux, uy, uz,
                                                            vx, vy, vz, hp, bx, by, bz, acc);
        }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        float h[8];
#pragma unroll
        for (int m = 0; m < 8; ++m) {
            const float2 t2 = f2_unpack(acc[j][m]);   // halves: even, odd atoms
            h[m] = t2.x + t2.y;
        }
        const float Kr = h[0], Ki = h[1], Rr = h[2], Ri = h[3];
        const float Sr = h[4], Si = h[5], Qr = h[6], Qi = h[7];
        // A(s, t) = K - s t Q + i t R + i s S
        csr[4 * j] = (Kr - Qr) + (Ri + Si);       // a (-, -)
        csi[4 * j] = (Ki - Qi) - (Rr + Sr);
        csr[4 * j + 1] = (Kr + Qr) + (Ri - Si);   // b (+, -)
        csi[4 * j + 1] = (Ki + Qi) - (Rr - Sr);
        csr[4 * j + 2] = (Kr + Qr) - (Ri - Si);   // c (-, +)
        csi[4 * j + 2] = (Ki + Qi) + (Rr - Sr);
        csr[4 * j + 3] = (Kr - Qr) - (Ri + Si);   // d (+, +)
        csi[4 * j + 3] = (Ki - Qi) + (Rr + Sr);
    }
}

// Tiles wider than the square form's radius: the square's four quads on
// their own, two at a time (the 2-quad loop; its register use stays below
// the square loop's).
template <bool CPLX>
__device__ __forceinline__ void mk_square_quads_tile(const MkSplitArgs &A, const mk_frame_desc &F,
                                                     const double4 &o, bool fr_tile,
                                                     const float4 *__restrict__ P,
                                                     const float4 *__restrict__ E, int T,
                                                     const float (&wx)[16], const float (&wy)[16],
                                                     const float (&wz)[16], const float (&hq)[16],
                                                     float (&csr)[16], float (&csi)[16])
{
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        float hx[8], hy[8], hz[8], hh[8], hr[8], hi[8];
#pragma unroll
        for (int p = 0; p < 8; ++p) {
            hx[p] = wx[8 * h + p]; hy[p] = wy[8 * h + p]; hz[p] = wz[8 * h + p]; hh[p] = hq[8 * h + p];
        }
        mk_quads_tile<2, CPLX>(A, F, o, fr_tile, P, E, T, hx, hy, hz, hh, hr, hi);
#pragma unroll
        for (int p = 0; p < 8; ++p) {
            csr[8 * h + p] = hr[p];
            csi[8 * h + p] = hi[p];
        }
    }
}

template <int NT, int PIX, bool FRESNEL, bool CPLX, int PM, bool ANA>
__global__ void __launch_bounds__(NT, (mk_min_blocks<NT, PIX, PM, ANA>()))
    mk_split_kernel(const __grid_constant__ MkSplitArgs A)
{
    extern __shared__ __align__(128) unsigned char smem[];
    const int T = A.tile_atoms;
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    long long *s_item = reinterpret_cast<long long *>(smem + 64);
    float4 *s_pos = reinterpret_cast<float4 *>(smem + 128);     // [2][T]
    float2 *s_amp = reinterpret_cast<float2 *>(s_pos + 2 * T);   // [2][T]
    // 8-pixel quad kernels keep each pixel's Kahan state (acc re, acc im,
    // comp re, comp im) in shared memory, [PIX][NT] float4, not in registers:
    // with it and w rebuilt in the fold they fit three 128-thread blocks per
    // SM (152 registers) instead of two (234); measured +2 % on the 8.19M-atom
    // step, while the 4-pixel kernels (126 registers already) lost 1.4 %.
    // The square kernels keep a compact state, 12 bytes a pixel: the two
    // sums as float2 and their Kahan compensations rounded to bfloat16
    // (8 significant bits of a term already below the sum's last bit, which
    // keeps the folds' sum good to ~2^-32 relative), so that three blocks fit
    // an SM with 1024-atom tiles (3 x (48 + 24) KB).
    constexpr bool KS = ((PM == 2 || PM == 3) && PIX == 8) || (PM == 4 && PIX == 16);
    constexpr bool KC = PM == 4;
    float4 *s_kahan = reinterpret_cast<float4 *>(s_amp + 2 * T);            // [PIX][NT]
    float2 *s_kacc = reinterpret_cast<float2 *>(s_amp + 2 * T);             // KC: [PIX][NT]
    __nv_bfloat162 *s_kcmp = reinterpret_cast<__nv_bfloat162 *>(s_kacc + PIX * NT);
    const int tid = threadIdx.x;
    const uint32_t tile_bytes = (uint32_t)T * (uint32_t)(sizeof(float4) + sizeof(float2));

    if (tid == 0) {
        mk_mbar_init(&bar[0], 1);
        mk_mbar_init(&bar[1], 1);
        mk_fence_barrier_init();
    }
    __syncthreads();
    unsigned it = 0;   // tiles consumed by this block: selects buffer and phase

    for (;;) {
        if (tid == 0) *s_item = (long long)atomicAdd(A.counter, 1ull);
        __syncthreads();
        const long long item = *s_item;
        __syncthreads();                    // s_item may be rewritten next round
        if (item >= A.n_items) break;

        // item -> (frame, pixel block, slice)
        int f = 0;
        if (A.n_frames > 1) {
            int lo = 0, hi = A.n_frames - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (A.frames[mid].item_off <= item) lo = mid; else hi = mid - 1;
            }
            f = lo;
        }
        const mk_frame_desc F = A.n_frames > 1 ? A.frames[f] : A.f0;
        const long long local = item - F.item_off;
        const int pb = (int)(local % F.pix_blocks);
        const int slice = (int)(local / F.pix_blocks);
        const int t_lo = slice * F.tiles_per_slice;
        const int t_hi = min(A.n_tiles, t_lo + F.tiles_per_slice);
        if (tid == 0) {
            mk_issue_tile(A, s_pos, s_amp, bar, it & 1, t_lo, T, tile_bytes);
            if (t_lo + 1 < t_hi) mk_issue_tile(A, s_pos, s_amp, bar, (it + 1) & 1, t_lo + 1, T, tile_bytes);
        }

        int pix[PIX];
        // squares: the thread's pixels from the square's first pixel and the
        // row length (two registers across the tile loop instead of 16)
        int sqb = 0, sqr = 0;
        auto pixat = [&](int p) -> int {
            if constexpr (PM == 4)
                return sqb >= F.n_pix ? F.n_pix
                                      : sqb + (2 * (p >> 3) + ((p >> 1) & 1)) * sqr +
                                            2 * ((p >> 2) & 1) + (p & 1);
            else
                return pix[p];
        };
        float accr[PIX], acci[PIX], cmpr[PIX], cmpi[PIX];
#pragma unroll
        for (int p = 0; p < PIX; ++p) {
            // pairs: pixels 2j, 2j+1 of the thread are detector neighbours
            // (consecutive indices; the host only pairs within rows)
            pix[p] = PM == 1 ? pb * (NT * PIX) + 2 * ((p >> 1) * NT + tid) + (p & 1)
                             : pb * (NT * PIX) + p * NT + tid;
            accr[p] = acci[p] = cmpr[p] = cmpi[p] = 0.f;
            if constexpr (KC) {
                s_kacc[p * NT + tid] = make_float2(0.f, 0.f);
                s_kcmp[p * NT + tid] = __floats2bfloat162_rn(0.f, 0.f);
            } else if constexpr (KS) {
                s_kahan[p * NT + tid] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
        // pixels this thread writes (a quad's repeated edge pixel is not)
        unsigned keep = (1u << PIX) - 1u;
        if constexpr (PM == 3) {
            // octet of the thread: rows 2 gz, 2 gz + 1, columns 4 gy .. 4 gy + 3;
            // pixels 0..3 = quad (a, b, c, d) at columns 4 gy, 4 gy + 1, pixels
            // 4..7 the quad at 4 gy + 2, 4 gy + 3. The planner admits only
            // frames of whole octets (row % 4 == 0, an even row count); past
            // the last octet the pixels get n_pix (loads clamp, stores skip).
            static_assert(PIX == 8, "octets are 8 pixels a thread");
            const int row = max(F.row, 1), rows = F.n_pix / row;
            const int gpr = row >> 2, n_oct = gpr * (rows >> 1);
            const int gi = pb * NT + tid;
            if (gi < n_oct) {
                const int gz = gi / gpr, gy = gi - gz * gpr;
                const int a0 = 2 * gz * row + 4 * gy, c0 = a0 + row;
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    pix[4 * j] = a0 + 2 * j;
                    pix[4 * j + 1] = a0 + 2 * j + 1;
                    pix[4 * j + 2] = c0 + 2 * j;
                    pix[4 * j + 3] = c0 + 2 * j + 1;
                }
            } else {
#pragma unroll
                for (int p = 0; p < PIX; ++p) pix[p] = F.n_pix;
            }
        }
        if constexpr (PM == 4) {
            // square of the thread: rows 4 gz .. 4 gz + 3, columns 4 gy ..
            // 4 gy + 3; quad j at rows 4 gz + 2 (j >> 1) (+1), columns
            // 4 gy + 2 (j & 1) (+1). The planner admits only frames of whole
            // squares (row % 4 == 0, row count % 4 == 0); past the last square
            // the pixels get n_pix (loads clamp, stores skip).
            static_assert(PIX == 16, "squares are 16 pixels a thread");
            const int row = max(F.row, 1), rows = F.n_pix / row;
            const int gpr = row >> 2, n_sq = gpr * (rows >> 2);
            const int gi = pb * NT + tid;
            sqr = row;
            sqb = F.n_pix;
            if (gi < n_sq) {
                const int gz = gi / gpr, gy = gi - gz * gpr;
                sqb = 4 * gz * row + 4 * gy;   // pixel 4j + e at sqb + pixat's offset
            }
        }
        if constexpr (PM == 2) {
            // quad j of the thread: pixels 4j..4j+3 = a, b (row 2 qz) and c, d
            // (row 2 qz + 1) at columns 2 qy, 2 qy + 1. An odd last column or
            // row repeats the edge pixel (u or v is then exactly 0) and only
            // its first copy is stored; out-of-range quads get n_pix (loads
            // clamp, stores skip).
            const int row = max(F.row, 1), rows = F.n_pix / row;
            const int half = (row + 1) >> 1, n_quads = half * ((rows + 1) >> 1);
#pragma unroll
            for (int j = 0; j < PIX / 4; ++j) {
                const int qi = pb * (NT * (PIX / 4)) + j * NT + tid;
                if (qi < n_quads) {
                    const int qz = qi / half, qy = qi - qz * half;
                    const int r0 = 2 * qz, c0 = 2 * qy;
                    const int r1 = min(r0 + 1, rows - 1), c1 = min(c0 + 1, row - 1);
                    pix[4 * j] = r0 * row + c0;
                    pix[4 * j + 1] = r0 * row + c1;
                    pix[4 * j + 2] = r1 * row + c0;
                    pix[4 * j + 3] = r1 * row + c1;
                    if (c1 == c0) keep &= ~(0xAu << (4 * j));   // b, d repeat a, c
                    if (r1 == r0) keep &= ~(0xCu << (4 * j));   // c, d repeat a, b
                } else {
                    pix[4 * j] = pix[4 * j + 1] = pix[4 * j + 2] = pix[4 * j + 3] = F.n_pix;
                }
            }
        }

        for (int t = t_lo; t < t_hi; ++t, ++it) {
            const int buf = it & 1;
            const uint32_t parity = (it >> 1) & 1u;
            const double4 o = A.origin[t];
            const float ox = (float)o.x, oy = (float)o.y, oz = (float)o.z;
            // Per (tile, pixel): w = b - u' in registers for the atom loop.
            float wx[PIX], wy[PIX], wz[PIX], hq[PIX];
#pragma unroll
            for (int p = 0; p < PIX; ++p) {
                const long long g = F.pix_off + min(pixat(p), F.n_pix - 1);
                const float4 uu = A.u[g];
                const float uo = fmaf(uu.z, oz, fmaf(uu.y, oy, uu.x * ox));
                wx[p] = F.b[0] - (uu.x - (ox - uo * uu.x) * uu.w);
                wy[p] = F.b[1] - (uu.y - (oy - uo * uu.y) * uu.w);
                wz[p] = F.b[2] - (uu.z - (oz - uo * uu.z) * uu.w);
                // 1 / (2 kappa |P - o|) for the |d|^2 term (D is in cycles).
                hq[p] = FRESNEL ? 0.5f * uu.w / (A.kappa * fmaf(-uo, uu.w, 1.f)) : 0.f;
            }
            // Analyser per (tile, pixel), in FP64: x0 = |u' - c|^2 at the tile
            // origin and its gradient in the offset D; a top-hat factor is one
            // number for the whole tile unless the tile's spread of x crosses
            // the acceptance edge.
            float agx[PIX], agy[PIX], agz[PIX], ath[PIX], ag0[PIX], ag1[PIX];
            bool warp_atom = false, warp_zero = false;
            if constexpr (ANA) {
                bool need_atom = false, all_zero = true;
#pragma unroll
                for (int p = 0; p < PIX; ++p) {
                    const long long g = F.pix_off + min(pixat(p), F.n_pix - 1);
                    const double4 qq = A.q[g];
                    const double ip = (double)A.u[g].w;
                    const double ux = A.an_b[0] - qq.x * A.inv_kappa;
                    const double uy = A.an_b[1] - qq.y * A.inv_kappa;
                    const double uz = A.an_b[2] - qq.z * A.inv_kappa;
                    const double uo = ux * o.x + uy * o.y + uz * o.z;
                    const double px_ = ux - (o.x - uo * ux) * ip;
                    const double py_ = uy - (o.y - uo * uy) * ip;
                    const double pz_ = uz - (o.z - uo * uz) * ip;
                    const double vx = px_ - A.an_c[0], vy = py_ - A.an_c[1], vz = pz_ - A.an_c[2];
                    const double x0 = vx * vx + vy * vy + vz * vz;
                    const double ro = ip / (1.0 - uo * ip);          // 1 / |P - o|
                    const double vu = vx * px_ + vy * py_ + vz * pz_;
                    const double gs = -2.0 * ro * A.inv_kappa;       // per cycle of D
                    const double gxd = gs * (vx - vu * px_), gyd = gs * (vy - vu * py_),
                                 gzd = gs * (vz - vu * pz_);
                    agx[p] = (float)gxd; agy[p] = (float)gyd; agz[p] = (float)gzd;
                    const double rho = o.w;
                    const double spread = sqrt(gxd * gxd + gyd * gyd + gzd * gzd) * rho / A.inv_kappa +
                                          4.0 * rho * rho * ro * ro;
                    ath[p] = INFINITY;
                    ag1[p] = 0.f;
                    if (A.analyser == 1) {
                        if (x0 + spread <= A.an_xacc) {
                            ag0[p] = 1.f;
                        } else if (x0 - spread > A.an_xacc) {
                            ag0[p] = 0.f;
                        } else {
                            ag0[p] = 1.f;
                            ath[p] = (float)(A.an_xacc - x0);
                            need_atom = true;
                        }
                    } else if (A.analyser == 2 && A.an_hw > 0.0) {
                        // G(x) = 1 / (1 + theta^2 / hw^2), theta = 2 asin(sqrt(x)/2);
                        // dtheta^2/dx = (theta / sqrt x) / sqrt(1 - x/4)
                        const double sx = sqrt(x0);
                        const double thv = 2.0 * asin(fmin(0.5 * sx, 1.0));
                        const double ts = sx > 1e-6 ? thv / sx : 1.0 + x0 / 24.0;
                        const double r = thv / A.an_hw;
                        const double G0 = 1.0 / (1.0 + r * r);
                        const double G1 = -G0 * G0 * ts / sqrt(fmax(1.0 - 0.25 * x0, 1e-30)) /
                                          (A.an_hw * A.an_hw);
                        ag0[p] = (float)G0;
                        ag1[p] = (float)G1;
                        need_atom = true;
                    } else {
                        ag0[p] = 1.f;
                    }
                    if (pixat(p) < F.n_pix && ag0[p] != 0.f) all_zero = false;
                }
                warp_atom = __any_sync(0xffffffffu, need_atom);
                warp_zero = __all_sync(0xffffffffu, all_zero && !need_atom);
            }
            const bool ok = mk_mbar_wait_bounded(&bar[buf], parity, MK_WAIT_LIMIT_NS);
            if (__syncthreads_or(!ok)) {
                if (tid == 0) {
                    atomicExch(A.status, MK_DEV_TIMEOUT_TMA);
                    // Let any copy still in flight land before the block's
                    // shared memory is released (bounded as well).
                    mk_mbar_wait_bounded(&bar[buf ^ 1], ((it + 1) >> 1) & 1u, MK_WAIT_LIMIT_NS / 2);
                }
                return;
            }
            const float4 *P = s_pos + buf * T;
            // T float2 amplitudes = T/2 float4 (interleaved atom pairs)
            const float4 *E = reinterpret_cast<const float4 *>(s_amp + buf * T);
            float csr[PIX], csi[PIX];
#pragma unroll
            for (int p = 0; p < PIX; ++p) csr[p] = csi[p] = 0.f;
            // The |d|^2 term only for tiles wide enough to need it (uniform
            // across the block: no divergence).
            const bool fr_tile = FRESNEL && (float)o.w > A.fres_r;
            // analyser: a warp whose pixels are all outside the acceptance
            // skips the tile; one with a pixel the acceptance edge cuts (or
            // any Darwin expansion) takes the per-atom loop; the rest run the
            // pixel-sharing form and take one factor per (tile, pixel) below
            const bool ana_skip = ANA && warp_zero, ana_atom = ANA && warp_atom && !warp_zero;
            if (ana_skip) {
            } else if (ana_atom) {
                if (fr_tile)
                    mk_tile_terms_ana<PIX, true, CPLX>(P, E, T, wx, wy, wz, hq, F.b[0], F.b[1], F.b[2],
                                                       agx, agy, agz, ath, ag0, ag1, csr, csi);
                else
                    mk_tile_terms_ana<PIX, false, CPLX>(P, E, T, wx, wy, wz, hq, F.b[0], F.b[1], F.b[2],
                                                        agx, agy, agz, ath, ag0, ag1, csr, csi);
            } else if constexpr (PM == 4) {
                // tiles wider than the square form's radius (the host bounds
                // its dropped phase per radius): the square's quads on their own
                if ((float)o.w > A.oct_r)
                    mk_square_quads_tile<CPLX>(A, F, o, fr_tile, P, E, T, wx, wy, wz, hq, csr, csi);
                else
                    mk_square_tile<CPLX>(A, F, o, fr_tile, P, E, T, wx, wy, wz, hq, csr, csi);
            } else if constexpr (PM == 3) {
                // tiles wider than the octet form's radius (the host bounds its
                // dropped phase per radius): the thread's two quads on their own
                if ((float)o.w > A.oct_r)
                    mk_quads_tile<2, CPLX>(A, F, o, fr_tile, P, E, T, wx, wy, wz, hq, csr, csi);
                else
                    mk_octet_tile<CPLX>(A, F, o, fr_tile, P, E, T, wx, wy, wz, hq, csr, csi);
            } else if constexpr (PM == 2) {
                mk_quads_tile<PIX / 4, CPLX>(A, F, o, fr_tile, P, E, T, wx, wy, wz, hq, csr, csi);
            } else if constexpr (PM == 1) {
                constexpr int NP = PIX / 2;
                mk_f2 sx[NP], sy[NP], sz[NP], dx[NP], dy[NP], dz[NP], hp[NP];
                mk_f2 pr[NP], pi_[NP], sr[NP], si[NP];
#pragma unroll
                for (int q = 0; q < NP; ++q) {
                    const int a = 2 * q, b = 2 * q + 1;
                    sx[q] = f2_splat(0.5f * (wx[a] + wx[b]));
                    sy[q] = f2_splat(0.5f * (wy[a] + wy[b]));
                    sz[q] = f2_splat(0.5f * (wz[a] + wz[b]));
                    dx[q] = f2_splat(3.14159265358979f * (wx[a] - wx[b]));
                    dy[q] = f2_splat(3.14159265358979f * (wy[a] - wy[b]));
                    dz[q] = f2_splat(3.14159265358979f * (wz[a] - wz[b]));
                    hp[q] = f2_splat(0.5f * (hq[a] + hq[b]));
                    pr[q] = pi_[q] = sr[q] = si[q] = 0ull;    // +0.0f in both halves
                }
                const mk_f2 bx = f2_splat(F.b[0]), by = f2_splat(F.b[1]), bz = f2_splat(F.b[2]);
                // the short delta polynomial for tiles small enough (uniform
                // across the block, like fr_tile)
                const bool short_tile = (float)o.w <= A.pair_short_r;
                if (fr_tile) {
                    if (short_tile)
                        mk_tile_terms_pair<NP, true, CPLX, true>(P, E, T, sx, sy, sz, dx, dy, dz, hp,
                                                                 bx, by, bz, pr, pi_, sr, si);
                    else
                        mk_tile_terms_pair<NP, true, CPLX, false>(P, E, T, sx, sy, sz, dx, dy, dz, hp,
                                                                  bx, by, bz, pr, pi_, sr, si);
                } else {
                    if (short_tile)
                        mk_tile_terms_pair<NP, false, CPLX, true>(P, E, T, sx, sy, sz, dx, dy, dz, hp,
                                                                  bx, by, bz, pr, pi_, sr, si);
                    else
                        mk_tile_terms_pair<NP, false, CPLX, false>(P, E, T, sx, sy, sz, dx, dy, dz, hp,
                                                                   bx, by, bz, pr, pi_, sr, si);
                }
#pragma unroll
                for (int q = 0; q < NP; ++q) {
                    // halves = even and odd atoms of the tile
                    const float2 a = f2_unpack(pr[q]), b = f2_unpack(pi_[q]);
                    const float2 c = f2_unpack(sr[q]), d = f2_unpack(si[q]);
                    const float P_re = a.x + a.y, P_im = b.x + b.y;
                    const float S_im = c.x + c.y, S_re = d.x + d.y;   // Q = i S
                    csr[2 * q] = P_re - S_im;
                    csi[2 * q] = P_im + S_re;
                    csr[2 * q + 1] = P_re + S_im;
                    csi[2 * q + 1] = P_im - S_re;
                }
            } else {
                if (fr_tile)
                    mk_tile_terms<PIX, true, CPLX>(P, E, T, wx, wy, wz, hq, F.b[0], F.b[1], F.b[2], csr, csi);
                else
                    mk_tile_terms<PIX, false, CPLX>(P, E, T, wx, wy, wz, hq, F.b[0], F.b[1], F.b[2], csr, csi);
            }
            if constexpr (ANA) {
                if (!ana_skip && !ana_atom) {
#pragma unroll
                    for (int p = 0; p < PIX; ++p) {   // one analyser factor per (tile, pixel)
                        csr[p] *= ag0[p];
                        csi[p] *= ag0[p];
                    }
                }
            }
            __syncthreads();   // every thread is done with buffer `buf`
            if (tid == 0 && t + 2 < t_hi) {
                mk_fence_proxy_async();
                mk_issue_tile(A, s_pos, s_amp, bar, buf, t + 2, T, tile_bytes);
            }
            // Fold: tile sum x factor x exp(2 pi i phi0), Kahan-compensated.
            // The square kernels read the tile origin again here rather
            // than keep it across the atom loop (registers).
            const int s = A.tspecies[t];
            const double4 of = PM == 4 ? mk_ld_origin(A.origin + t) : o;
            const float fox = PM == 4 ? (float)of.x : ox, foy = PM == 4 ? (float)of.y : oy,
                        foz = PM == 4 ? (float)of.z : oz;
            const float oo = fmaf(foz, foz, fmaf(foy, foy, fox * fox));
#pragma unroll
            for (int p = 0; p < PIX; ++p) {
                const long long g = F.pix_off + min(pixat(p), F.n_pix - 1);
                const float4 uu = KS ? mk_ld_fold(A.u + g) : A.u[g];
                const double4 qq = A.q[g];
                const float uo = fmaf(uu.z, foz, fmaf(uu.y, foy, uu.x * fox));
                const double q0 = qq.x * of.x + qq.y * of.y + qq.z * of.z;
                float ph = (float)(q0 - rint(q0)) + A.kappa * 0.5f * fmaf(-uo, uo, oo) * uu.w;
                ph -= rintf(ph);
                float s0, c0;
                __sincosf(ph * TWO_PI_F, &s0, &c0);
                float fx = wx[p], fy = wy[p], fz = wz[p];
                if constexpr (KS && !ANA) {   // w again, from the fresh load
                    fx = F.b[0] - (uu.x - (fox - uo * uu.x) * uu.w);
                    fy = F.b[1] - (uu.y - (foy - uo * uu.y) * uu.w);
                    fz = F.b[2] - (uu.z - (foz - uo * uu.z) * uu.w);
                }
                float2 Fc;
                if (A.ftab) {   // warp-uniform: a kernel argument
                    Fc = A.ftab[(long long)s * A.ftab_n + g];
                    if (A.decay) {
                        const float dr = 1.f / fmaf(-uo, uu.w, 1.f);
                        Fc.x *= dr;
                        Fc.y *= dr;
                    }
                } else {
                    Fc = mk_factor(A, s, F, fx, fy, fz, (float)qq.w, 1.f / fmaf(-uo, uu.w, 1.f));
                }
                const float gr = Fc.x * c0 - Fc.y * s0, gi = Fc.x * s0 + Fc.y * c0;
                const float tr = csr[p] * gr - csi[p] * gi;
                const float ti = csr[p] * gi + csi[p] * gr;
                float ar = accr[p], ai = acci[p], kr = cmpr[p], ki = cmpi[p];
                if constexpr (KC) {
                    const float2 a2 = s_kacc[p * NT + tid];
                    const __nv_bfloat162 c2 = s_kcmp[p * NT + tid];
                    ar = a2.x; ai = a2.y; kr = __low2float(c2); ki = __high2float(c2);
                } else if constexpr (KS) {
                    const float4 k4 = s_kahan[p * NT + tid];
                    ar = k4.x; ai = k4.y; kr = k4.z; ki = k4.w;
                }
                float y = tr - kr;
                float z = ar + y;
                kr = (z - ar) - y;
                ar = z;
                y = ti - ki;
                z = ai + y;
                ki = (z - ai) - y;
                ai = z;
                if constexpr (KC) {
                    s_kacc[p * NT + tid] = make_float2(ar, ai);
                    s_kcmp[p * NT + tid] = __floats2bfloat162_rn(kr, ki);
                } else if constexpr (KS) {
                    s_kahan[p * NT + tid] = make_float4(ar, ai, kr, ki);
                } else {
                    accr[p] = ar; acci[p] = ai; cmpr[p] = kr; cmpi[p] = ki;
                }
            }
        }
#pragma unroll
        for (int p = 0; p < PIX; ++p) {
            if constexpr (KC) {
                const float2 a2 = s_kacc[p * NT + tid];
                const __nv_bfloat162 c2 = s_kcmp[p * NT + tid];
                accr[p] = a2.x; acci[p] = a2.y; cmpr[p] = __low2float(c2); cmpi[p] = __high2float(c2);
            } else if constexpr (KS) {
                const float4 k4 = s_kahan[p * NT + tid];
                accr[p] = k4.x; acci[p] = k4.y; cmpr[p] = k4.z; cmpi[p] = k4.w;
            }
            if (pixat(p) < F.n_pix && ((keep >> p) & 1u))
                A.partial[F.part_off + (long long)slice * F.n_pix + pixat(p)] =
                    make_double2((double)accr[p] - (double)cmpr[p], (double)acci[p] - (double)cmpi[p]);
        }
    }
}

// ----------------------------------------------------------------- pickers
typedef void (*mk_split_fn)(const MkSplitArgs);

template <int NT, int PIX, int PM, bool ANA>
static mk_split_fn mk_pick4(bool fresnel, bool cplx)
{
    if (fresnel)
        return cplx ? mk_split_kernel<NT, PIX, true, true, PM, ANA>
                    : mk_split_kernel<NT, PIX, true, false, PM, ANA>;
    return cplx ? mk_split_kernel<NT, PIX, false, true, PM, ANA>
                : mk_split_kernel<NT, PIX, false, false, PM, ANA>;
}

// Pairs need an even PIX; the analyser kernels (no pairs) exist for
// 128/256 threads and 2 or 4 pixels per thread.
template <int NT, int PIX>
static mk_split_fn mk_pick3(bool fresnel, bool cplx, bool pair, bool ana)
{
    if (ana) {
        if constexpr ((NT == 128 || NT == 256) && (PIX == 2 || PIX == 4))
            return pair ? nullptr : mk_pick4<NT, PIX, 0, true>(fresnel, cplx);
        return nullptr;
    }
    if constexpr (PIX % 2 == 0) {
        if (pair) return mk_pick4<NT, PIX, 1, false>(fresnel, cplx);
    } else {
        if (pair) return nullptr;
    }
    return mk_pick4<NT, PIX, 0, false>(fresnel, cplx);
}

// Kernel instance for a launch shape of one block size (nullptr when no
// instance exists); defined in mk_split_k<NT>.cu.
mk_split_fn mk_pick_nt64(int pix, bool fresnel, bool cplx, bool pair, bool ana);
mk_split_fn mk_pick_nt128(int pix, bool fresnel, bool cplx, bool pair, bool ana);
mk_split_fn mk_pick_nt256(int pix, bool fresnel, bool cplx, bool pair, bool ana);
// Pixel-quad instances (64/128/256 threads, 4 or 8 pixels a thread; with the
// analyser 128/256 threads); defined in mk_split_quad.cu, mk_split_quad8.cu
// and mk_split_quad_ana.cu.
mk_split_fn mk_pick_quad(int nt, int pix, bool fresnel, bool cplx, bool ana);
// Pixel-octet instances (64/128/256 threads, 8 pixels a thread, no
// analyser); defined in mk_split_oct.cu.
mk_split_fn mk_pick_oct(int nt, int pix, bool fresnel, bool cplx, bool ana);
// Pixel-square instances (128 or 192 threads, 16 pixels a thread, no
// analyser); defined in mk_split_sq.cu and mk_split_sq192.cu.
mk_split_fn mk_pick_sq(int nt, int pix, bool fresnel, bool cplx, bool ana);

#define MK_PIX_CASES(NT_)                                                  \
    switch (pix) {                                                         \
    case 1: return mk_pick3<NT_, 1>(fresnel, cplx, pair, ana);             \
    case 2: return mk_pick3<NT_, 2>(fresnel, cplx, pair, ana);             \
    case 4: return mk_pick3<NT_, 4>(fresnel, cplx, pair, ana);             \
    case 8: return mk_pick3<NT_, 8>(fresnel, cplx, pair, ana);             \
    default: return nullptr;                                               \
    }
