// Staging kernels: per-pixel prologue, stage transform + incident amplitude,
// species-partitioned Morton order and atom tiles with FP64 origins.
#include <cub/device/device_radix_sort.cuh>

#include "mk_common.cuh"

// ------------------------------------------------------------------ pixels
// One thread per pixel. Everything of magnitude |P| is kept in double here so
// the sum kernels only ever see it as (i) an FP64 dot product with a tile
// origin and (ii) the per-pixel phasor exp(i k |P|).
__global__ void mk_pixels_kernel(int ny, int nz, const double *__restrict__ xyz, double kappa,
                                 double k, double bx, double by, double bz, double *__restrict__ r0,
                                 double4 *__restrict__ q, float4 *__restrict__ u,
                                 double2 *__restrict__ phasor)
{
    const int n = ny * nz;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const double tx = xyz[3 * p], ty = xyz[3 * p + 1], tz = xyz[3 * p + 2];
    const double R = sqrt(tx * tx + ty * ty + tz * tz);
    double ux = 0.0, uy = 0.0, uz = 0.0;
    if (R > 0.0) { ux = tx / R; uy = ty / R; uz = tz / R; }
    r0[p] = R;
    u[p] = make_float4((float)ux, (float)uy, (float)uz, R > 0.0 ? (float)(1.0 / R) : 0.f);
    double s, c;
    sincos(fmod(k * R, MK_TWO_PI), &s, &c);
    phasor[p] = make_double2(c, s);
    // Q_cut: half the pixel diagonal in Q from the right and upper neighbours,
    // edge pixels taking the inner one (compute_scattering_cffi, Beam.py:716-746).
    const int col = p % ny, row = p / ny;
    const int nb0 = (col + 1 < ny) ? p + 1 : ((col > 0) ? p - 1 : p);
    const int nb1 = (row + 1 < nz) ? p + ny : ((row > 0) ? p - ny : p);
    double q2 = 0.0;
    for (int j = 0; j < 2; ++j) {
        const int m = j ? nb1 : nb0;
        const double rx = xyz[3 * m], ry = xyz[3 * m + 1], rz = xyz[3 * m + 2];
        const double Rr = sqrt(rx * rx + ry * ry + rz * rz);
        double cd = (Rr > 0.0) ? (ux * rx + uy * ry + uz * rz) / Rr : 1.0;
        cd = fmin(1.0, fmax(-1.0, cd));
        const double qn = k * sqrt(fmax(0.0, 2.0 * (1.0 - cd)));
        q2 += qn * qn;
    }
    q[p] = make_double4(kappa * (bx - ux), kappa * (by - uy), kappa * (bz - uz), 0.5 * sqrt(q2));
}

extern "C" int mk_pixels_prepare(const mk_pixels *px, const mk_physics *phys, void *stream)
{
    MK_REQUIRE(px && phys, "mk_pixels_prepare: null argument");
    MK_REQUIRE(px->ny > 0 && px->nz > 0, "mk_pixels_prepare: empty detector (%d x %d)", px->ny, px->nz);
    MK_REQUIRE(px->xyz && px->r0 && px->q && px->u && px->phasor,
               "mk_pixels_prepare: null pixel buffer");
    MK_REQUIRE(phys->k > 0.0, "mk_pixels_prepare: k must be positive");
    const int64_t n = (int64_t)px->ny * px->nz;
    MK_REQUIRE(n < (1ll << 31), "mk_pixels_prepare: too many pixels");
    const double kappa = phys->k / MK_TWO_PI;
    const int th = 256;
    mk_pixels_kernel<<<(unsigned)((n + th - 1) / th), th, 0, mk_stream(stream)>>>(
        px->ny, px->nz, px->xyz, kappa, phys->k, phys->beam_dir[0], phys->beam_dir[1],
        phys->beam_dir[2], px->r0, reinterpret_cast<double4 *>(px->q),
        reinterpret_cast<float4 *>(px->u), reinterpret_cast<double2 *>(px->phasor));
    MK_CHECK_CUDA(cudaGetLastError());
    return MK_OK;
}

// ------------------------------------------------- stage transform + E_in
// float32 lab position r = R p + t with separately rounded products and sums
// (no contraction), then E0 sampled bilinearly at (u, v) = (y, z) with the
// reference's float32 arithmetic; 0 outside the grid (Beam.py:956-1045).
struct MkRot {
    float r[9];
    float t[3];
    double grid[4];
};

__global__ void mk_atoms_lab_kernel(int64_t n, const float *__restrict__ pin, MkRot R,
                                    const float2 *__restrict__ e0, int gny, int gnz,
                                    double *__restrict__ pos_lab, float2 *__restrict__ amp)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x = pin[3 * i], y = pin[3 * i + 1], z = pin[3 * i + 2];
    float l[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        float acc = __fmul_rn(x, R.r[3 * r]);
        acc = __fadd_rn(acc, __fmul_rn(y, R.r[3 * r + 1]));
        acc = __fadd_rn(acc, __fmul_rn(z, R.r[3 * r + 2]));
        l[r] = __fadd_rn(acc, R.t[r]);
    }
    pos_lab[3 * i] = __ddiv_rn((double)l[0], 1e10);
    pos_lab[3 * i + 1] = __ddiv_rn((double)l[1], 1e10);
    pos_lab[3 * i + 2] = __ddiv_rn((double)l[2], 1e10);
    float2 a = make_float2(1.f, 0.f);
    if (e0) {
        const float iu = __fadd_rn(__fdiv_rn(l[1], (float)R.grid[0]), (float)R.grid[2]);
        const float iv = __fadd_rn(__fdiv_rn(l[2], (float)R.grid[1]), (float)R.grid[3]);
        a = make_float2(0.f, 0.f);
        if (iu >= 0.f && iu <= (float)(gny - 1) && iv >= 0.f && iv <= (float)(gnz - 1)) {
            const int i0 = (int)floorf(iu), j0 = (int)floorf(iv);
            const int i1 = min(i0 + 1, gny - 1), j1 = min(j0 + 1, gnz - 1);
            const float fu = __fsub_rn(iu, (float)i0), fv = __fsub_rn(iv, (float)j0);
            const float gu = __fsub_rn(1.f, fu), gv = __fsub_rn(1.f, fv);
            const float w00 = __fmul_rn(gu, gv), w01 = __fmul_rn(gu, fv);
            const float w10 = __fmul_rn(fu, gv), w11 = __fmul_rn(fu, fv);
            const float2 e00 = e0[i0 * gnz + j0], e01 = e0[i0 * gnz + j1];
            const float2 e10 = e0[i1 * gnz + j0], e11 = e0[i1 * gnz + j1];
            float re = __fmul_rn(e00.x, w00), im = __fmul_rn(e00.y, w00);
            re = __fadd_rn(re, __fmul_rn(e01.x, w01));
            im = __fadd_rn(im, __fmul_rn(e01.y, w01));
            re = __fadd_rn(re, __fmul_rn(e10.x, w10));
            im = __fadd_rn(im, __fmul_rn(e10.y, w10));
            re = __fadd_rn(re, __fmul_rn(e11.x, w11));
            im = __fadd_rn(im, __fmul_rn(e11.y, w11));
            a = make_float2(re, im);
        }
    }
    amp[i] = a;
}

extern "C" int mk_atoms_lab(int64_t n, const float *pos_in, const float *rot, const float *trans,
                            const float *e0, int grid_ny, int grid_nz, const double *grid,
                            double *pos_lab, float *amp, void *stream)
{
    MK_REQUIRE(n >= 0, "mk_atoms_lab: negative atom count");
    if (n == 0) return MK_OK;
    MK_REQUIRE(pos_in && rot && trans && pos_lab && amp, "mk_atoms_lab: null argument");
    MK_REQUIRE(!e0 || (grid && grid_ny > 0 && grid_nz > 0 && grid[0] > 0.0 && grid[1] > 0.0),
               "mk_atoms_lab: beam grid needs positive sizes and spacings");
    MkRot R;
    for (int i = 0; i < 9; ++i) R.r[i] = rot[i];
    for (int i = 0; i < 3; ++i) R.t[i] = trans[i];
    for (int i = 0; i < 4; ++i) R.grid[i] = grid ? grid[i] : 1.0;
    const int th = 256;
    mk_atoms_lab_kernel<<<(unsigned)((n + th - 1) / th), th, 0, mk_stream(stream)>>>(
        n, pos_in, R, reinterpret_cast<const float2 *>(e0), grid_ny, grid_nz, pos_lab,
        reinterpret_cast<float2 *>(amp));
    MK_CHECK_CUDA(cudaGetLastError());
    return MK_OK;
}

// ------------------------------------------------------------- tiles
// Bounding box of all atoms (for the Morton quantisation): one block-level
// min/max per block, combined with atomics on the ordered-integer image of
// the doubles.
__device__ __forceinline__ unsigned long long mk_ordered(double v)
{
    const unsigned long long b = __double_as_longlong(v);
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double mk_unordered(unsigned long long o)
{
    const unsigned long long b = (o & 0x8000000000000000ull) ? (o & ~0x8000000000000000ull) : ~o;
    return __longlong_as_double(b);
}

__global__ void mk_bbox_init(unsigned long long *bb)
{
    if (threadIdx.x < 3) bb[threadIdx.x] = ~0ull;       // min
    else if (threadIdx.x < 6) bb[threadIdx.x] = 0ull;   // max
}

__global__ void mk_bbox_kernel(int64_t n, const double *__restrict__ pos, unsigned long long *bb)
{
    unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0ull, 0ull, 0ull};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const unsigned long long o = mk_ordered(pos[3 * i + c]);
            lo[c] = o < lo[c] ? o : lo[c];
            hi[c] = o > hi[c] ? o : hi[c];
        }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        for (int off = 16; off > 0; off >>= 1) {
            const unsigned long long a = __shfl_xor_sync(0xffffffffu, lo[c], off);
            const unsigned long long b = __shfl_xor_sync(0xffffffffu, hi[c], off);
            lo[c] = a < lo[c] ? a : lo[c];
            hi[c] = b > hi[c] ? b : hi[c];
        }
        if ((threadIdx.x & 31) == 0) {
            atomicMin(&bb[c], lo[c]);
            atomicMax(&bb[3 + c], hi[c]);
        }
    }
}

// Position along a 3-D Hilbert curve of 2^19 cells per axis (the
// axes-to-transpose construction of J. Skilling, "Programming the Hilbert
// curve", AIP Conf. Proc. 707, 381 (2004)): undo the rotations/reflections
// level by level, Gray-encode, then read the bits out MSB first, x first.
// Unlike a Z-order (Morton) curve, consecutive cells are always face
// neighbours, so a run of consecutive atoms never spans two distant corners
// of the sample and every tile stays compact.
#define MK_HILBERT_BITS 17   // per axis inside one cube: 51 bits
#define MK_MAX_CUBES 128     // 7 bits of cube index
#define MK_KEY_BITS 62       // + 4 bits of species (MK_MAX_SPECIES = 16)

__device__ __forceinline__ unsigned long long mk_hilbert3(uint32_t x, uint32_t y, uint32_t z)
{
    uint32_t X[3] = {x, y, z};
    for (uint32_t Q = 1u << (MK_HILBERT_BITS - 1); Q > 1; Q >>= 1) {
        const uint32_t P = Q - 1;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            if (X[i] & Q) {
                X[0] ^= P;
            } else {
                const uint32_t t = (X[0] ^ X[i]) & P;
                X[0] ^= t;
                X[i] ^= t;
            }
        }
    }
    X[1] ^= X[0];
    X[2] ^= X[1];
    uint32_t t = 0;
    for (uint32_t Q = 1u << (MK_HILBERT_BITS - 1); Q > 1; Q >>= 1)
        if (X[2] & Q) t ^= Q - 1;
    X[0] ^= t;
    X[1] ^= t;
    X[2] ^= t;
    unsigned long long h = 0;
    for (int b = MK_HILBERT_BITS - 1; b >= 0; --b) {
        h = (h << 1) | ((X[0] >> b) & 1u);
        h = (h << 1) | ((X[1] >> b) & 1u);
        h = (h << 1) | ((X[2] >> b) & 1u);
    }
    return h;
}

// Sort key: species in bits 58..61, then a row of cubes, then the Hilbert
// index inside the atom's cube. The bounding box is cut into cubes whose
// side is its shortest extent (enlarged until at most MK_MAX_CUBES), taken
// x fastest. The curve runs from a cube's (0,0,0) corner to its (max,0,0)
// corner, so consecutive cubes along x join without a jump; only row ends
// do. One cube size for all axes keeps tiles round, and filling every cube
// keeps the curve out of empty space (where its excursions would put
// far-apart atoms next to each other in the order).
__global__ void mk_keys_kernel(int64_t n, const double *__restrict__ pos,
                               const int *__restrict__ species,
                               const unsigned long long *__restrict__ bb,
                               unsigned long long *__restrict__ keys, int *__restrict__ idx)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double lo[3], span[3], side = 0.0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        lo[c] = mk_unordered(bb[c]);
        span[c] = mk_unordered(bb[3 + c]) - lo[c];
        if (span[c] > 0.0 && (side == 0.0 || span[c] < side)) side = span[c];
    }
    if (!(side > 0.0)) side = 1.0;
    int nc[3];
    for (;;) {
#pragma unroll
        for (int c = 0; c < 3; ++c) nc[c] = max(1, (int)ceil(span[c] / side - 1e-9));
        if (nc[0] * nc[1] * nc[2] <= MK_MAX_CUBES) break;
        side *= 1.25;
    }
    uint32_t q[3];
    int cube[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const double t = (pos[3 * i + c] - lo[c]) / side;
        cube[c] = min(nc[c] - 1, max(0, (int)floor(t)));
        const double f = fmin(fmax(t - cube[c], 0.0), 1.0);
        q[c] = (uint32_t)(f * (double)((1u << MK_HILBERT_BITS) - 1));
    }
    const unsigned long long ci = (unsigned long long)((cube[2] * nc[1] + cube[1]) * nc[0] + cube[0]);
    keys[i] = ((unsigned long long)species[i] << 58) | (ci << 51) | mk_hilbert3(q[0], q[1], q[2]);
    idx[i] = (int)i;
}

struct MkTileMap {
    int n_species;
    int tile_atoms;
    long long run_start[MK_MAX_SPECIES];  // first sorted index of each species
    long long run_count[MK_MAX_SPECIES];
    int tile_start[MK_MAX_SPECIES + 1];   // first tile of each species
};

// One block per tile: gather its atoms in sorted order, FP64 bounding-box
// centre as origin, offsets k/2pi (a - o) rounded once to float32.
template <int NT>
__global__ void __launch_bounds__(NT) mk_tile_kernel(MkTileMap M, double kappa,
                                                      const double *__restrict__ pos,
                                                      const float2 *__restrict__ amp,
                                                      const int *__restrict__ order,
                                                      double4 *__restrict__ origin,
                                                      int *__restrict__ tspecies,
                                                      float4 *__restrict__ tpos,
                                                      float2 *__restrict__ tamp)
{
    const int t = blockIdx.x;
    int s = 0;
    while (s + 1 < M.n_species && t >= M.tile_start[s + 1]) ++s;
    const long long first = M.run_start[s] + (long long)(t - M.tile_start[s]) * M.tile_atoms;
    const long long end = M.run_start[s] + M.run_count[s];
    __shared__ double red[6][NT / 32];
    __shared__ double org[3];
    __shared__ double rad2[NT / 32];

    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int j = threadIdx.x; j < M.tile_atoms; j += NT) {
        const long long si = first + j;
        if (si < end) {
            const int a = order[si];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const double v = pos[3 * (long long)a + c];
                lo[c] = fmin(lo[c], v);
                hi[c] = fmax(hi[c], v);
            }
        }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        for (int off = 16; off > 0; off >>= 1) {
            lo[c] = fmin(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], off));
            hi[c] = fmax(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], off));
        }
        if ((threadIdx.x & 31) == 0) {
            red[c][threadIdx.x >> 5] = lo[c];
            red[3 + c][threadIdx.x >> 5] = hi[c];
        }
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double l = 1e300, h = -1e300;
        for (int w = 0; w < NT / 32; ++w) {
            l = fmin(l, red[threadIdx.x][w]);
            h = fmax(h, red[3 + threadIdx.x][w]);
        }
        org[threadIdx.x] = 0.5 * (l + h);
    }
    __syncthreads();
    const double ox = org[0], oy = org[1], oz = org[2];
    double r2max = 0.0;
    const long long base = (long long)t * M.tile_atoms;
    for (int j = threadIdx.x; j < M.tile_atoms; j += NT) {
        const long long si = first + j;
        float4 P = make_float4(0.f, 0.f, 0.f, 0.f);
        float2 E = make_float2(0.f, 0.f);
        if (si < end) {
            const int a = order[si];
            const double dx = pos[3 * (long long)a] - ox;
            const double dy = pos[3 * (long long)a + 1] - oy;
            const double dz = pos[3 * (long long)a + 2] - oz;
            const double d2 = dx * dx + dy * dy + dz * dz;
            r2max = fmax(r2max, d2);
            P = make_float4((float)(kappa * dx), (float)(kappa * dy), (float)(kappa * dz),
                            (float)(kappa * kappa * d2));
            E = amp[a];
        }
        // atom pairs interleaved: per pair (2q, 2q+1) the floats
        // x0 x1 y0 y1 z0 z1 w0 w1 and er0 er1 ei0 ei1, so that the sum
        // kernels load two atoms' coordinates as packed f32x2 operands
        float *pf = reinterpret_cast<float *>(tpos) + 4 * (base + (j & ~1));
        float *af = reinterpret_cast<float *>(tamp) + 2 * (base + (j & ~1));
        const int h = j & 1;
        pf[h] = P.x;
        pf[2 + h] = P.y;
        pf[4 + h] = P.z;
        pf[6 + h] = P.w;
        af[h] = E.x;
        af[2 + h] = E.y;
    }
    for (int off = 16; off > 0; off >>= 1) r2max = fmax(r2max, __shfl_xor_sync(0xffffffffu, r2max, off));
    if ((threadIdx.x & 31) == 0) rad2[threadIdx.x >> 5] = r2max;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = 0.0;
        for (int w = 0; w < NT / 32; ++w) m = fmax(m, rad2[w]);
        origin[t] = make_double4(ox, oy, oz, sqrt(m));
        tspecies[t] = s;
    }
}

static size_t mk_align256(size_t b) { return (b + 255) & ~(size_t)255; }

static size_t mk_cub_temp_bytes(int64_t n)
{
    size_t tb = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tb, (unsigned long long *)nullptr,
                                    (unsigned long long *)nullptr, (int *)nullptr, (int *)nullptr,
                                    (int)n, 0, MK_KEY_BITS);
    return tb;
}

extern "C" size_t mk_tiles_workspace_size(int64_t n)
{
    if (n <= 0) return 256;
    return mk_align256(64) + 2 * mk_align256(8 * (size_t)n) + 2 * mk_align256(4 * (size_t)n) +
           mk_align256(mk_cub_temp_bytes(n));
}

extern "C" int mk_tiles_build(int64_t n, const double *pos, const int *species, const float *amp,
                              int n_species, const int64_t *counts, double k, mk_tiles *tiles,
                              void *workspace, size_t ws_bytes, void *stream)
{
    MK_REQUIRE(tiles && counts, "mk_tiles_build: null argument");
    MK_REQUIRE(n_species >= 1 && n_species <= MK_MAX_SPECIES, "mk_tiles_build: 1..%d species",
               MK_MAX_SPECIES);
    MK_REQUIRE(n > 0 && n < (1ll << 31), "mk_tiles_build: atom count %lld out of range",
               (long long)n);
    MK_REQUIRE(pos && species && amp && tiles->origin && tiles->species && tiles->pos && tiles->amp,
               "mk_tiles_build: null buffer");
    const int T = tiles->tile_atoms;
    MK_REQUIRE(T >= 128 && T <= 4096 && (T & (T - 1)) == 0,
               "mk_tiles_build: tile_atoms must be a power of two in [128, 4096]");
    MkTileMap M;
    memset(&M, 0, sizeof(M));
    M.n_species = n_species;
    M.tile_atoms = T;
    long long run = 0, total = 0;
    int tiles_needed = 0;
    for (int s = 0; s < n_species; ++s) {
        MK_REQUIRE(counts[s] >= 0, "mk_tiles_build: negative count");
        M.run_start[s] = run;
        M.run_count[s] = counts[s];
        M.tile_start[s] = tiles_needed;
        run += counts[s];
        tiles_needed += (int)((counts[s] + T - 1) / T);
        total += counts[s];
    }
    M.tile_start[n_species] = tiles_needed;
    MK_REQUIRE(total == n, "mk_tiles_build: species counts sum to %lld, expected %lld", total,
               (long long)n);
    MK_REQUIRE(tiles->n_tiles == tiles_needed, "mk_tiles_build: n_tiles %d, layout needs %d",
               tiles->n_tiles, tiles_needed);
    const size_t need = mk_tiles_workspace_size(n);
    if (!workspace || ws_bytes < need) {
        mk_set_error("mk_tiles_build: workspace %zu bytes, need %zu", ws_bytes, need);
        return MK_ENOMEM;
    }
    char *w = static_cast<char *>(workspace);
    unsigned long long *bb = reinterpret_cast<unsigned long long *>(w);
    w += mk_align256(64);
    unsigned long long *k_in = reinterpret_cast<unsigned long long *>(w);
    w += mk_align256(8 * (size_t)n);
    unsigned long long *k_out = reinterpret_cast<unsigned long long *>(w);
    w += mk_align256(8 * (size_t)n);
    int *i_in = reinterpret_cast<int *>(w);
    w += mk_align256(4 * (size_t)n);
    int *i_out = reinterpret_cast<int *>(w);
    w += mk_align256(4 * (size_t)n);
    size_t temp = mk_cub_temp_bytes(n);
    cudaStream_t st = mk_stream(stream);

    mk_bbox_init<<<1, 32, 0, st>>>(bb);
    const int th = 256;
    const int nb = (int)std::min<int64_t>((n + th - 1) / th, 4096);
    mk_bbox_kernel<<<nb, th, 0, st>>>(n, pos, bb);
    mk_keys_kernel<<<(unsigned)((n + th - 1) / th), th, 0, st>>>(n, pos, species, bb, k_in, i_in);
    MK_CHECK_CUDA(cudaGetLastError());
    MK_CHECK_CUDA(cub::DeviceRadixSort::SortPairs(w, temp, k_in, k_out, i_in, i_out, (int)n, 0,
                                                  MK_KEY_BITS, st));
    if (tiles_needed > 0) {
        mk_tile_kernel<256><<<tiles_needed, 256, 0, st>>>(
            M, k / MK_TWO_PI, pos, reinterpret_cast<const float2 *>(amp), i_out,
            reinterpret_cast<double4 *>(tiles->origin), tiles->species,
            reinterpret_cast<float4 *>(tiles->pos), reinterpret_cast<float2 *>(tiles->amp));
        MK_CHECK_CUDA(cudaGetLastError());
    }
    return MK_OK;
}
