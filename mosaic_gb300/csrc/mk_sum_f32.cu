// FP32 split-phase kinematic sum over Hilbert-ordered atom tiles (sm_103a),
// one persistent kernel for single exposures and batched scans.
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
#include <climits>
#include <algorithm>
#include <mutex>

#include "mk_split.cuh"

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

// out[g] (+)= scale * phasor[g] * sum_s partial[frame][s][p]: the slices of
// every pixel added in order in FP64; frames found by binary search.
__global__ void mk_reduce_kernel(const double2 *__restrict__ partial, long long n_total,
                                 int n_frames, mk_frame_desc f0,
                                 const mk_frame_desc *__restrict__ frames,
                                 const double2 *__restrict__ phasor, double scale,
                                 double2 *__restrict__ out, int accumulate)
{
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n_total) return;
    int f = 0;
    if (n_frames > 1) {
        int lo = 0, hi = n_frames - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (frames[mid].pix_off <= g) lo = mid; else hi = mid - 1;
        }
        f = lo;
    }
    const mk_frame_desc F = n_frames > 1 ? frames[f] : f0;
    const long long p = g - F.pix_off;
    double re = 0.0, im = 0.0;
    for (int s = 0; s < F.slices; ++s) {
        const double2 v = partial[F.part_off + (long long)s * F.n_pix + p];
        re += v.x;
        im += v.y;
    }
    if (phasor) {
        const double2 e = phasor[g];
        const double r2 = re * e.x - im * e.y, i2 = re * e.y + im * e.x;
        re = r2;
        im = i2;
    }
    re *= scale;
    im *= scale;
    if (accumulate) {
        const double2 o = out[g];
        re += o.x;
        im += o.y;
    }
    out[g] = make_double2(re, im);
}

// sums[f] = sum over the frame's pixels of |A|^2, one block per frame,
// fixed-order tree reduction.
__global__ void mk_frame_intensity_kernel(const double2 *__restrict__ field, int n_frames,
                                          const mk_frame_desc *__restrict__ frames, mk_frame_desc f0,
                                          double *__restrict__ sums)
{
    __shared__ double red[256];
    const int f = blockIdx.x;
    const mk_frame_desc F = n_frames > 1 ? frames[f] : f0;
    double acc = 0.0;
    for (int p = threadIdx.x; p < F.n_pix; p += blockDim.x) {
        const double2 v = field[F.pix_off + p];
        acc += v.x * v.x + v.y * v.y;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) sums[f] = red[0];
}

int mk_launch_reduce(const double2 *partial, int slices, int n_pix, const double2 *phasor,
                     double scale, double2 *out, int accumulate, cudaStream_t st)
{
    mk_frame_desc F;
    memset(&F, 0, sizeof(F));
    F.n_pix = n_pix;
    F.slices = slices;
    mk_reduce_kernel<<<(n_pix + 255) / 256, 256, 0, st>>>(partial, n_pix, 1, F, nullptr, phasor,
                                                          scale, out, accumulate);
    MK_CHECK_CUDA(cudaGetLastError());
    return MK_OK;
}

// ----------------------------------------------------------------- launch
static mk_split_fn mk_pick(int nt, int pix, bool fresnel, bool cplx, int pair, bool ana)
{
    if (pair == 4) return mk_pick_sq(nt, pix, fresnel, cplx, ana);
    if (pair == 3) return mk_pick_oct(nt, pix, fresnel, cplx, ana);
    if (pair == 2) return mk_pick_quad(nt, pix, fresnel, cplx, ana);
    switch (nt) {
    case 64: return mk_pick_nt64(pix, fresnel, cplx, pair, ana);
    case 128: return mk_pick_nt128(pix, fresnel, cplx, pair, ana);
    case 256: return mk_pick_nt256(pix, fresnel, cplx, pair, ana);
    default: return nullptr;
    }
}

// Two tile buffers; 8-pixel quad and octet kernels add their per-pixel
// Kahan state (16 bytes a pixel), square kernels their compact one (12).
static size_t mk_split_smem(int T, const mk_launch *launch)
{
    size_t b = 128 + (size_t)2 * T * (sizeof(float4) + sizeof(float2));
    if ((launch->pairs == 2 || launch->pairs == 3) && launch->pix_per_thread == 8)
        b += sizeof(float4) * (size_t)launch->pix_per_thread * launch->threads;
    if (launch->pairs == 4 && launch->pix_per_thread == 16)
        b += (sizeof(float2) + 4) * (size_t)launch->pix_per_thread * launch->threads;
    return b;
}

struct MkLaunchShape {
    mk_split_fn fn;
    int resident;      // blocks that fit the GPU at once
};

static int mk_launch_shape(int tile_atoms, const mk_launch *launch, MkLaunchShape *out,
                           bool ana = false)
{
    mk_split_fn fn = mk_pick(launch->threads, launch->pix_per_thread, launch->fresnel != 0,
                             launch->amp_real == 0, launch->pairs, ana);
    MK_REQUIRE(fn, "split kernel: unsupported launch shape threads=%d pix=%d pairs=%d%s",
               launch->threads, launch->pix_per_thread, launch->pairs,
               ana ? " with the analyser (128/256 threads; 2/4 pixels, or quads with 4/8; no pairs)"
                   : (launch->pairs == 2 ? " (quads: 4 or 8 pixels a thread)"
                      : launch->pairs == 3 ? " (octets: 8 pixels a thread, no analyser)"
                      : launch->pairs == 4 ? " (squares: 16 pixels, 128 or 192 threads, no analyser)"
                                           : ""));
    const size_t smem = mk_split_smem(tile_atoms, launch);
    MK_CHECK_CUDA(cudaFuncSetAttribute((const void *)fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
    int dev = 0, sms = 0, bps = 0;
    MK_CHECK_CUDA(cudaGetDevice(&dev));
    MK_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    MK_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, (const void *)fn,
                                                                launch->threads, smem));
    MK_REQUIRE(bps >= 1, "split kernel: launch shape does not fit on an SM");
    out->fn = fn;
    out->resident = sms * bps;
    return MK_OK;
}

// Slice count for one frame so that the items fill the resident grid many
// times over (load balance) while keeping items long enough that the
// per-item TMA pipeline start is negligible.
static int mk_frame_slices(int pix_blocks, int n_tiles, int resident, long long total_blocks)
{
    const long long target = 24LL * resident;
    long long s = (target + total_blocks - 1) / std::max<long long>(total_blocks, 1);
    s = std::max<long long>(1, std::min<long long>(s, std::max(1, n_tiles / 4)));
    return (int)std::min<long long>(s, n_tiles);
}

extern "C" int mk_scan_plan(int n_frames, const int *frame_pixels, const int *frame_rows,
                            const double *beam_dirs, const double *pol_es, const mk_tiles *tiles,
                            const mk_launch *launch, mk_frame_desc *frames_out,
                            long long *n_items_out, long long *n_partial_out)
{
    MK_REQUIRE(n_frames >= 1 && frame_pixels && beam_dirs && tiles && launch && frames_out &&
                   n_items_out && n_partial_out,
               "mk_scan_plan: null argument or no frames");
    MK_REQUIRE(tiles->n_tiles >= 1, "mk_scan_plan: no tiles");
    MK_REQUIRE(launch->pairs >= 0 && launch->pairs <= 4,
               "mk_scan_plan: pairs must be 0, 1, 2, 3 or 4");
    if (launch->pairs >= 2) {
        MK_REQUIRE(frame_rows, "mk_scan_plan: pixel quads, octets and squares need the row length of every frame");
        for (int f = 0; f < n_frames; ++f)
            MK_REQUIRE(frame_rows[f] >= 1 && frame_pixels[f] % frame_rows[f] == 0,
                       "mk_scan_plan: frame %d: %d pixels are not whole rows of %d",
                       f, frame_pixels[f], frame_rows[f]);
    }
    if (launch->pairs == 3) {
        for (int f = 0; f < n_frames; ++f)
            MK_REQUIRE(frame_rows[f] % 4 == 0 && (frame_pixels[f] / frame_rows[f]) % 2 == 0,
                       "mk_scan_plan: frame %d (%d x %d pixels) is not whole 2x4 octets: rows of a "
                       "multiple of 4 pixels and an even row count are needed",
                       f, frame_rows[f], frame_pixels[f] / frame_rows[f]);
    }
    if (launch->pairs == 4) {
        for (int f = 0; f < n_frames; ++f)
            MK_REQUIRE(frame_rows[f] % 4 == 0 && (frame_pixels[f] / frame_rows[f]) % 4 == 0,
                       "mk_scan_plan: frame %d (%d x %d pixels) is not whole 4x4 squares: rows of a "
                       "multiple of 4 pixels and a row count that is a multiple of 4 are needed",
                       f, frame_rows[f], frame_pixels[f] / frame_rows[f]);
    }
    MkLaunchShape sh;
    int rc = mk_launch_shape(tiles->tile_atoms, launch, &sh);
    if (rc != MK_OK) return rc;
    const int ppb = launch->threads * launch->pix_per_thread;
    // pixel slots of a frame: quads round both sides up to even (the odd
    // edge repeats its pixels); octets and squares tile the frame exactly
    auto slots = [&](int f) -> long long {
        if (launch->pairs != 2) return frame_pixels[f];
        const long long row = frame_rows[f], rows = frame_pixels[f] / row;
        return 4LL * ((row + 1) / 2) * ((rows + 1) / 2);
    };
    long long total_blocks = 0;
    for (int f = 0; f < n_frames; ++f) {
        MK_REQUIRE(frame_pixels[f] >= 1, "mk_scan_plan: frame %d has no pixels", f);
        total_blocks += (slots(f) + ppb - 1) / ppb;
    }
    long long pix_off = 0, part_off = 0, item_off = 0;
    for (int f = 0; f < n_frames; ++f) {
        mk_frame_desc &F = frames_out[f];
        memset(&F, 0, sizeof(F));
        F.n_pix = frame_pixels[f];
        F.row = frame_rows ? frame_rows[f] : 0;
        F.pix_blocks = (int)((slots(f) + ppb - 1) / ppb);
        int s = launch->slices > 0 ? std::min(launch->slices, tiles->n_tiles)
                                   : mk_frame_slices(F.pix_blocks, tiles->n_tiles, sh.resident, total_blocks);
        F.tiles_per_slice = (tiles->n_tiles + s - 1) / s;
        F.slices = (tiles->n_tiles + F.tiles_per_slice - 1) / F.tiles_per_slice;
        F.pix_off = pix_off;
        F.part_off = part_off;
        F.item_off = item_off;
        for (int c = 0; c < 3; ++c) {
            F.b[c] = (float)beam_dirs[3 * f + c];
            F.e[c] = pol_es ? (float)pol_es[3 * f + c] : 0.f;
        }
        pix_off += F.n_pix;
        part_off += (long long)F.slices * F.n_pix;
        item_off += (long long)F.slices * F.pix_blocks;
    }
    *n_items_out = item_off;
    *n_partial_out = part_off;
    return MK_OK;
}

extern "C" size_t mk_scan_workspace_size(long long n_partial)
{
    return 256 + sizeof(double2) * (size_t)std::max<long long>(n_partial, 1);
}

static int mk_run_split(const mk_tiles *tiles, const mk_species *spc, const mk_physics *phys,
                        const mk_pixels *px, long long n_total, int n_frames,
                        const mk_frame_desc &f0, const mk_frame_desc *frames_dev,
                        long long n_items, long long n_partial, const mk_launch *launch,
                        double *out, double *sums, int accumulate, void *workspace,
                        size_t ws_bytes, cudaStream_t st)
{
    MK_REQUIRE(px->q && px->u && px->phasor, "split kernel: pixels not prepared");
    MK_REQUIRE(tiles->origin && tiles->species && tiles->pos && tiles->amp,
               "split kernel: null tile buffer");
    MK_REQUIRE(((uintptr_t)tiles->pos & 15) == 0 && ((uintptr_t)tiles->amp & 15) == 0,
               "split kernel: tile arrays must be 16-byte aligned");
    const int T = tiles->tile_atoms;
    MK_REQUIRE(T >= 128 && T <= 4096 && (T & (T - 1)) == 0, "split kernel: bad tile_atoms %d", T);
    const size_t need = mk_scan_workspace_size(n_partial);
    if (!workspace || ws_bytes < need) {
        mk_set_error("split kernel: workspace %zu bytes, need %zu", ws_bytes, need);
        return MK_ENOMEM;
    }
    MkSplitArgs A;
    memset(&A, 0, sizeof(A));
    int rc = mk_species_pack(spc, &A.sp);
    if (rc != MK_OK) return rc;
    const bool ana = phys->analyser != 0;
    MK_REQUIRE(!ana || n_frames == 1, "split kernel: the analyser is for single exposures");
    MkLaunchShape sh;
    rc = mk_launch_shape(T, launch, &sh, ana);
    if (rc != MK_OK) return rc;
    mk_register_status_reader(mk_split_read_status);
    int *status = nullptr;
    MK_CHECK_CUDA(cudaGetSymbolAddress((void **)&status, g_split_status));
    char *w = static_cast<char *>(workspace);
    A.counter = reinterpret_cast<unsigned long long *>(w);
    A.partial = reinterpret_cast<double2 *>(w + 256);
    A.n_tiles = tiles->n_tiles;
    A.tile_atoms = T;
    A.n_frames = n_frames;
    A.n_items = n_items;
    A.f0 = f0;
    A.frames = frames_dev;
    A.q = reinterpret_cast<const double4 *>(px->q);
    A.u = reinterpret_cast<const float4 *>(px->u);
    A.origin = reinterpret_cast<const double4 *>(tiles->origin);
    A.tspecies = tiles->species;
    A.tpos = reinterpret_cast<const float4 *>(tiles->pos);
    A.tamp = reinterpret_cast<const float2 *>(tiles->amp);
    A.status = status;
    A.kappa = (float)(phys->k / MK_TWO_PI);
    A.k = (float)phys->k;
    const double sf = phys->k * 0.25e-10 / MK_PI;
    A.s2fac = (float)(sf * sf);
    A.apply_pol = phys->apply_pol;
    A.decay = phys->spherical_decay;
    A.remove_forward = phys->remove_forward;
    A.pdeg = (float)phys->pol_deg;
    A.fres_r = launch->fresnel_radius_m > 0.0 ? (float)launch->fresnel_radius_m : 0.f;
    A.pair_short_r = launch->pair_short_radius_m > 0.0 ? (float)launch->pair_short_radius_m : -1.f;
    A.oct_r = launch->octet_radius_m > 0.0 ? (float)launch->octet_radius_m : -1.f;
    MK_REQUIRE(!(px->factor && phys->remove_forward),
               "split kernel: a factor table cannot serve remove_forward (its Q < Q_cut test is "
               "per tile and pixel)");
    A.ftab = reinterpret_cast<const float2 *>(px->factor);
    A.ftab_n = n_total;
    A.sin_direct = launch->sin_direct_max_rad == 0.0 ? MK_SIN_DIRECT_MAX
                   : launch->sin_direct_max_rad < 0.0 ? -1.f : (float)launch->sin_direct_max_rad;
    if (ana) {
        double cx, cy, cz;
        rc = mk_analyser_pack(phys, &A.analyser, &cx, &cy, &cz, &A.an_xacc, &A.an_hw);
        if (rc != MK_OK) return rc;
        A.an_c[0] = cx; A.an_c[1] = cy; A.an_c[2] = cz;
        for (int c = 0; c < 3; ++c) A.an_b[c] = phys->beam_dir[c];
        A.inv_kappa = MK_TWO_PI / phys->k;
    }
    MK_CHECK_CUDA(cudaMemsetAsync(A.counter, 0, sizeof(unsigned long long), st));
    const long long grid = std::min<long long>(n_items, sh.resident);
    sh.fn<<<(unsigned)grid, launch->threads, mk_split_smem(T, launch), st>>>(A);
    MK_CHECK_CUDA(cudaGetLastError());
    const unsigned rb = (unsigned)((n_total + 255) / 256);
    mk_reduce_kernel<<<rb, 256, 0, st>>>(A.partial, n_total, n_frames, f0, frames_dev,
                                         reinterpret_cast<const double2 *>(px->phasor), MK_R_E,
                                         reinterpret_cast<double2 *>(out), accumulate);
    MK_CHECK_CUDA(cudaGetLastError());
    if (sums) {
        mk_frame_intensity_kernel<<<n_frames, 256, 0, st>>>(reinterpret_cast<const double2 *>(out),
                                                            n_frames, frames_dev, f0, sums);
        MK_CHECK_CUDA(cudaGetLastError());
    }
    return MK_OK;
}

// ------------------------------------------------------ factor table
// The scattering factor of every species at every pixel's own direction
// u (w = b - u), in the kernels' float32 arithmetic (mk_factor), without the
// spherical-decay ratio, which the split kernel applies per (tile, pixel).
__global__ void mk_factor_table_kernel(const __grid_constant__ MkSplitArgs A, long long n_pix,
                                       float2 *__restrict__ out)
{
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n_pix) return;
    int f = 0;
    if (A.n_frames > 1) {
        int lo = 0, hi = A.n_frames - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (A.frames[mid].pix_off <= g) lo = mid; else hi = mid - 1;
        }
        f = lo;
    }
    const mk_frame_desc F = A.n_frames > 1 ? A.frames[f] : A.f0;
    const float4 uu = A.u[g];
    const float qcut = (float)A.q[g].w;
    const float wx = F.b[0] - uu.x, wy = F.b[1] - uu.y, wz = F.b[2] - uu.z;
    for (int s = 0; s < A.sp.n; ++s) out[(long long)s * n_pix + g] = mk_factor(A, s, F, wx, wy, wz, qcut, 1.f);
}

extern "C" int mk_factor_table(const mk_pixels *px, const mk_species *spc, const mk_physics *phys,
                               int n_frames, const mk_frame_desc *frames_dev, void *stream)
{
    MK_REQUIRE(px && spc && phys, "mk_factor_table: null argument");
    MK_REQUIRE(px->factor && px->u && px->q, "mk_factor_table: pixels not prepared or no factor buffer");
    MK_REQUIRE(px->ny > 0 && px->nz > 0, "mk_factor_table: bad detector shape");
    MK_REQUIRE(phys->k > 0.0, "mk_factor_table: k must be positive");
    MK_REQUIRE(!phys->remove_forward,
               "mk_factor_table: remove_forward needs the factor per (tile, pixel)");
    MK_REQUIRE(n_frames <= 1 || frames_dev, "mk_factor_table: %d frames and no frame table", n_frames);
    MK_REQUIRE(((uintptr_t)px->factor & 7) == 0, "mk_factor_table: factor buffer must be 8-byte aligned");
    MkSplitArgs A;
    memset(&A, 0, sizeof(A));
    int rc = mk_species_pack(spc, &A.sp);
    if (rc != MK_OK) return rc;
    const long long n = (long long)px->ny * px->nz;
    A.n_frames = n_frames > 1 ? n_frames : 1;
    A.frames = frames_dev;
    A.f0.n_pix = (int)std::min<long long>(n, INT_MAX);
    for (int c = 0; c < 3; ++c) {
        A.f0.b[c] = (float)phys->beam_dir[c];
        A.f0.e[c] = (float)phys->pol_e[c];
    }
    A.q = reinterpret_cast<const double4 *>(px->q);
    A.u = reinterpret_cast<const float4 *>(px->u);
    A.k = (float)phys->k;
    const double sf = phys->k * 0.25e-10 / MK_PI;
    A.s2fac = (float)(sf * sf);
    A.apply_pol = phys->apply_pol;
    A.pdeg = (float)phys->pol_deg;
    cudaStream_t st = mk_stream(stream);
    mk_factor_table_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
        A, n, reinterpret_cast<float2 *>(px->factor));
    MK_CHECK_CUDA(cudaGetLastError());
    return MK_OK;
}

static int mk_single_plan(const mk_tiles *tiles, const mk_physics *phys, const mk_pixels *px,
                          const mk_launch *launch, mk_frame_desc *F, long long *n_items,
                          long long *n_partial)
{
    const int n_pix = px->ny * px->nz;
    return mk_scan_plan(1, &n_pix, &px->ny, phys->beam_dir, phys->pol_e, tiles, launch, F, n_items,
                        n_partial);
}

extern "C" int mk_split_plan(const mk_tiles *tiles, const mk_pixels *px, const mk_launch *launch,
                             size_t *ws_bytes_out)
{
    MK_REQUIRE(tiles && px && launch && ws_bytes_out, "mk_split_plan: null argument");
    MK_REQUIRE(px->ny > 0 && px->nz > 0, "mk_split_plan: bad detector shape");
    if (tiles->n_tiles <= 0) {
        *ws_bytes_out = mk_scan_workspace_size(0);
        return MK_OK;
    }
    mk_physics ph;
    memset(&ph, 0, sizeof(ph));
    ph.beam_dir[0] = 1.0;
    mk_frame_desc F;
    long long ni, np;
    int rc = mk_single_plan(tiles, &ph, px, launch, &F, &ni, &np);
    if (rc != MK_OK) return rc;
    *ws_bytes_out = mk_scan_workspace_size(np);
    return MK_OK;
}

extern "C" int mk_kin_split_f32(const mk_tiles *tiles, const mk_species *spc,
                                const mk_physics *phys, const mk_pixels *px,
                                const mk_launch *launch, double *out, int accumulate,
                                void *workspace, size_t ws_bytes, void *stream)
{
    MK_REQUIRE(tiles && spc && phys && px && launch && out, "mk_kin_split_f32: null argument");
    const int64_t np64 = (int64_t)px->ny * px->nz;
    MK_REQUIRE(px->ny > 0 && px->nz > 0 && np64 < (1ll << 31), "mk_kin_split_f32: bad detector shape");
    MK_REQUIRE(phys->k > 0.0, "mk_kin_split_f32: k must be positive");
    cudaStream_t st = mk_stream(stream);
    if (tiles->n_tiles <= 0) {
        if (!accumulate) MK_CHECK_CUDA(cudaMemsetAsync(out, 0, sizeof(double2) * (size_t)np64, st));
        return MK_OK;
    }
    mk_frame_desc F;
    long long n_items, n_partial;
    int rc = mk_single_plan(tiles, phys, px, launch, &F, &n_items, &n_partial);
    if (rc != MK_OK) return rc;
    return mk_run_split(tiles, spc, phys, px, np64, 1, F, nullptr, n_items, n_partial, launch, out,
                        nullptr, accumulate, workspace, ws_bytes, st);
}

// ------------------------------------------------------ allocation-free entry
// Scratch of mk_kin_split_f32_noalloc: one fixed array in every GPU that
// loads this library, held until the process exits. Its device address is
// looked up on the first call on each device (with that device current) and
// kept: host code cannot use the symbol itself, which on the host names a
// shadow object, not device memory. A cudaDeviceReset invalidates the kept
// address (the header says so).
static __device__ __align__(256) unsigned char g_noalloc_scratch[MK_NOALLOC_SCRATCH_BYTES];

static std::mutex g_noalloc_mu;
static void *g_noalloc_addr[256];

static int mk_noalloc_scratch(void **out)
{
    int dev = 0;
    MK_CHECK_CUDA(cudaGetDevice(&dev));
    MK_REQUIRE(dev >= 0 && dev < 256, "mk_kin_split_f32_noalloc: device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            mk_set_error("mk_kin_split_f32_noalloc: cannot resolve the scratch array on device %d: %s",
                         dev, cudaGetErrorString(e));
            return MK_ECUDA;
        }
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return MK_OK;
}

extern "C" int mk_kin_split_f32_noalloc(const mk_tiles *tiles, const mk_species *spc,
                                        const mk_physics *phys, const mk_pixels *px,
                                        const mk_launch *launch, double *out, int accumulate,
                                        void *stream)
{
    MK_REQUIRE(tiles && spc && phys && px && launch && out,
               "mk_kin_split_f32_noalloc: null argument");
    const int64_t np64 = (int64_t)px->ny * px->nz;
    MK_REQUIRE(px->ny > 0 && px->nz > 0 && np64 < (1ll << 31),
               "mk_kin_split_f32_noalloc: bad detector shape");
    MK_REQUIRE(phys->k > 0.0, "mk_kin_split_f32_noalloc: k must be positive");
    // Even one slice needs 16 bytes per pixel of partial field.
    const long long max_partial = (long long)((MK_NOALLOC_SCRATCH_BYTES - 256) / sizeof(double2));
    if (np64 > max_partial) {
        mk_set_error("mk_kin_split_f32_noalloc: %lld pixels need %lld bytes of scratch, more than "
                     "the fixed %u bytes; use mk_kin_split_f32 with a workspace",
                     (long long)np64, 256 + 16 * (long long)np64, (unsigned)MK_NOALLOC_SCRATCH_BYTES);
        return MK_ENOMEM;
    }
    cudaStream_t st = mk_stream(stream);
    if (tiles->n_tiles <= 0) {
        if (!accumulate) MK_CHECK_CUDA(cudaMemsetAsync(out, 0, sizeof(double2) * (size_t)np64, st));
        return MK_OK;
    }
    void *scratch = nullptr;
    int rc = mk_noalloc_scratch(&scratch);
    if (rc != MK_OK) return rc;
    mk_frame_desc F;
    long long n_items, n_partial;
    rc = mk_single_plan(tiles, phys, px, launch, &F, &n_items, &n_partial);
    if (rc != MK_OK) return rc;
    // Fewer slices when the partial fields would not fit the array; the plan
    // and the launch then both use the capped shape.
    mk_launch capped = *launch;
    const mk_launch *eff = launch;
    if (n_partial > max_partial) {
        capped.slices = (int)std::max<long long>(1, max_partial / np64);
        eff = &capped;
        rc = mk_single_plan(tiles, phys, px, eff, &F, &n_items, &n_partial);
        if (rc != MK_OK) return rc;
        MK_REQUIRE(n_partial <= max_partial,
                   "mk_kin_split_f32_noalloc: %lld partial entries exceed the fixed scratch",
                   n_partial);
    }
    return mk_run_split(tiles, spc, phys, px, np64, 1, F, nullptr, n_items, n_partial, eff, out,
                        nullptr, accumulate, scratch, MK_NOALLOC_SCRATCH_BYTES, st);
}

extern "C" int mk_kin_scan_f32(const mk_tiles *tiles, const mk_species *spc,
                               const mk_physics *phys, const mk_pixels *px, int n_frames,
                               const mk_frame_desc *frames_dev, long long n_items,
                               long long n_partial, const mk_launch *launch, double *out,
                               double *intensity_sums, void *workspace, size_t ws_bytes,
                               void *stream)
{
    MK_REQUIRE(tiles && spc && phys && px && launch && out && frames_dev,
               "mk_kin_scan_f32: null argument");
    MK_REQUIRE(n_frames >= 1 && n_items >= 1 && n_partial >= 1, "mk_kin_scan_f32: empty plan");
    MK_REQUIRE(tiles->n_tiles >= 1, "mk_kin_scan_f32: no tiles");
    MK_REQUIRE(phys->k > 0.0, "mk_kin_scan_f32: k must be positive");
    const long long n_total = (long long)px->ny * px->nz;
    mk_frame_desc dummy;
    memset(&dummy, 0, sizeof(dummy));
    if (n_frames == 1) {
        // a one-frame plan still lives on the device; the kernel then needs
        // it by value: read it back once (not capturable, so scans pass >1)
        MK_CHECK_CUDA(cudaMemcpy(&dummy, frames_dev, sizeof(dummy), cudaMemcpyDeviceToHost));
    }
    return mk_run_split(tiles, spc, phys, px, n_total, n_frames, dummy,
                        n_frames > 1 ? frames_dev : nullptr, n_items, n_partial, launch, out,
                        intensity_sums, 0, workspace, ws_bytes, mk_stream(stream));
}
