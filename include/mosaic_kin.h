/*
 * mosaic_kin.h -- C ABI of the GB300 (sm_103a) kinematic scattering library
 * libmosaic_kin.so.
 *
 * The library computes, for every detector pixel P, the near-field kinematic
 * sum of the MOSAIC reference (Beam.py:663-816, the per-term arithmetic of
 * `compute_scattering_cffi`):
 *
 *   A(P) = r_e sum_a E_in(a) [f0_s(Q) + f'_s + i f''_s] [exp(-B_s s^2)]
 *          [sqrt(Pol)] [R0/r] exp(i k (b.a + |P - a|))
 *
 * with b the incident direction (+x in the lab frame). Two kernels:
 *   - mk_kin_plain_f64: the FP64 direct sum, term for term as the reference
 *     CPU kernel (drop-in and on-device oracle);
 *   - mk_kin_split_f32: the FP32 split-phase sum over Hilbert-ordered atom
 *     tiles with FP64 tile origins, Kahan-compensated across tiles and an
 *     FP64 cross-slice reduction.
 *
 * Conventions
 *   - Every pointer documented as "device" is a CUDA device pointer owned by
 *     the caller; "host" pointers are read during the call only.
 *   - Pixel index p = iz * ny + iy (Detector.py:204-214).
 *   - Calls are stream-ordered on `stream` (a cudaStream_t, NULL = default)
 *     and return before the GPU work finishes; mk_sync_status() waits and
 *     reports device-side errors.
 *   - Return value: MK_OK or a negative MK_E* code; mk_last_error() gives a
 *     message (thread-local). Nothing aborts, exits or traps.
 *   - Scratch: entry points that need scratch take a `workspace` of at least
 *     the bytes the matching *_workspace_size() query returns.
 */
#ifndef MOSAIC_KIN_H
#define MOSAIC_KIN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MK_OK 0
#define MK_EINVAL (-1)   /* bad argument (the reference raises ValueError) */
#define MK_ENOMEM (-2)   /* workspace too small (the reference raises MemoryError) */
#define MK_ETIMEOUT (-3) /* a bounded device-side wait ran out */
#define MK_EDECLINE (-4) /* the FP32 path cannot meet its error budget here */
#define MK_ECUDA (-5)    /* CUDA runtime error */

#define MK_MAX_SPECIES 16

/* Per-species scattering data (host arrays, n_species <= MK_MAX_SPECIES).
 * Replaces the per-atom tables the reference builds in
 * cpu_scatter_chunk_cffi (Beam.py:5671-5691) and _species_rows
 * (Beam.py:1345-1357). */
typedef struct {
    int n_species;
    const float *wk;       /* (S, 11) Waasmaier-Kirfel a1..a5 c b1..b5 */
    const float *f0_zero;  /* (S) f0 at Q = 0 */
    const float *anom_re;  /* (S) f'  at the beam energy */
    const float *anom_im;  /* (S) f'' at the beam energy */
    const float *dw_b;     /* (S) Debye-Waller B [A^2]; NULL = no factor */
} mk_species;

/* Physics switches, the flags of compute_scattering_cffi (Beam.py:631-651). */
typedef struct {
    double k;             /* 2 pi / lambda [1/m] */
    double beam_dir[3];   /* unit incident direction in the frame of atoms and pixels */
    int apply_pol;        /* multiply by sqrt(P_pol) */
    double pol_deg;       /* degree of linear polarization p */
    double pol_e[3];      /* its unit vector (same frame) */
    int spherical_decay;  /* multiply by R0 / r */
    int remove_forward;   /* subtract f(0) where Q < Q_cut(pixel) */
    /* Analyser acceptance of the general kernel (Beam.py:2350-2378): with
     * theta the angle between the atom->pixel direction and the analyser
     * axis, 1: top-hat, factor 1 for theta <= analyser_accept and 0 beyond;
     * 2: Darwin roll-off 1 / (1 + (theta / analyser_halfwidth)^2) (factor 1
     * when the half-width is <= 0); 0: no analyser. */
    int analyser;
    double analyser_dir[3];     /* unit analyser axis (frame of atoms and pixels) */
    double analyser_accept;     /* top-hat acceptance half-angle [rad] */
    double analyser_halfwidth;  /* Darwin half-width [rad] */
} mk_physics;

/* Per-pixel derived data, device arrays of length n_pix, filled by
 * mk_pixels_prepare (replaces the per-pixel prologue of Beam.py:716-746 and
 * pixel_phasor, Beam.py:9241-9255). */
typedef struct {
    int ny, nz;           /* detector (or ROI) shape; n_pix = ny * nz */
    const double *xyz;    /* device (n_pix, 3) pixel coordinates [m] */
    double *r0;           /* device (n_pix) |P| */
    double *q;            /* device (n_pix, 4): (k / 2 pi)(b - u_hat) [cycles/m], Q_cut [1/m] */
    float *u;             /* device (n_pix, 4): u_hat (x, y, z) and 1/|P| as float */
    double *phasor;       /* device (n_pix, 2) exp(i k |P|) */
    float *factor;        /* device (n_species, n_pix, 2) or NULL: the scattering factor
                             (f0 + f' + i f'') e^{-B s^2} sqrt(P_pol) of every species at every
                             pixel's own direction, filled by mk_factor_table; the split kernels
                             then read it instead of evaluating the factor per (tile, pixel) */
} mk_pixels;

/* One frame of a batched launch (an exposure's pixels, or a scan step's
 * ROI), as filled by mk_scan_plan and read by the kernel from device
 * memory. The frames' pixels are consecutive in one set of mk_pixels
 * arrays; b and e are the incident direction and polarization vector in the
 * frame of the atoms (the sample frame for scans). 80 bytes. */
typedef struct {
    long long pix_off;    /* first pixel of the frame in the concatenated pixel arrays */
    long long part_off;   /* first entry of its partial fields in the workspace */
    long long item_off;   /* first work item of the frame */
    int n_pix;            /* pixels in the frame */
    int slices;           /* tile ranges summed separately (FP64 reduction) */
    int tiles_per_slice;
    int pix_blocks;       /* ceil(pixel slots / (threads * pix_per_thread)); slots = n_pix,
                             or with quads 4 ceil(row/2) ceil(rows/2) */
    float b[3];
    float e[3];
    int row;              /* pixels per detector row (0: unknown; pixel quads need it) */
    int reserved[3];
} mk_frame_desc;

/* Atom tiles for the split-phase kernel, filled by mk_tiles_build. Tiles
 * hold `tile_atoms` atoms of one species (the last tile of a species is
 * padded with zero-amplitude atoms). */
typedef struct {
    int n_tiles;
    int tile_atoms;       /* power of two, 128..4096 */
    double *origin;       /* device (n_tiles, 4): origin x, y, z [m], radius [m] */
    int *species;         /* device (n_tiles) species index */
    float *pos;           /* device (n_tiles*tile_atoms, 4): k/2pi (a - o) [cycles], |.|^2,
                             atom pairs interleaved: x0 x1 y0 y1 z0 z1 w0 w1 */
    float *amp;           /* device (n_tiles*tile_atoms, 2): incident amplitude,
                             atom pairs interleaved: re0 re1 im0 im1 */
} mk_tiles;

/* Launch shape of the split-phase kernel (autotuned by the host). */
typedef struct {
    int pix_per_thread;   /* 1, 2, 4 or 8; 16 with squares */
    int threads;          /* 64, 128 or 256; 128 or 192 with squares */
    int slices;           /* tile ranges summed separately, reduced in FP64; <= 0: auto */
    int fresnel;          /* 1: keep the |d|^2 term of the in-tile distance; 0: drop it
                             (the caller checks k r_tile^2 / 2 R0_min against its budget);
                             -1: keep it */
    int amp_real;         /* 1: every incident amplitude is real (skips two FMAs a term) */
    double fresnel_radius_m; /* with fresnel != 0: only tiles whose radius exceeds this keep
                                the |d|^2 term (0: every tile) */
    int pairs;            /* 1: pixels 2j, 2j+1 of every frame share one MUFU sin/cos (their
                             phase difference on FMA-pipe polynomials); the caller checks that
                             the half difference pi |D| |w_a - w_b| stays below 0.5 rad for
                             every tile (pix_per_thread even).
                             2: 2x2 pixel quads (two neighbours in a row and the two below
                             them) share one sin/cos; the two half differences along the row
                             and across rows go to polynomials and the quad's mixed second
                             difference (pi/2) D.(w_a + w_d - w_b - w_c) is dropped: the caller
                             checks the half differences as for pairs and the dropped term
                             against its phase budget (pix_per_thread 4 or 8; an odd last
                             column or row repeats its pixels inside the quad).
                             3: 2x4 pixel octets (see octet_radius_m).
                             4: 4x4 pixel squares (see octet_radius_m) */
    double pair_short_radius_m; /* with pairs, quads, octets or squares: tiles up to this radius keep the half
                             differences below 0.07 rad and use the short polynomials
                             (0: none does) */
    double sin_direct_max_rad; /* with quads, octets or squares: tiles without the |d|^2 term whose
                             in-tile phase bound stays below this [rad] pass the phase to the
                             MUFU sin/cos without the mod-1 reduction (its error grows
                             ~1e-7 |x|); 0: the library default, 100 rad; < 0: never */
    double octet_radius_m; /* with octets (pairs 3: two quads side by side in a 2x4 block share
                             their half differences, pix_per_thread 8, frames of whole octets):
                             tiles up to this radius [m] take the octet form, wider ones the
                             quad form; the caller bounds the octet's dropped phase (the
                             departure of w from a plane over the 8 pixels, times k r) for
                             that radius; <= 0: every tile takes the quad form.
                             With squares (pairs 4: four quads in a 4x4 block share their half
                             differences, pix_per_thread 16, 128 or 192 threads, frames of whole
                             squares: a row length and a row count that are multiples of 4)
                             the same for the square form and the departure of w from a plane
                             over its 16 pixels */
} mk_launch;

/* --- library ---------------------------------------------------------- */
int mk_version(void);
const char *mk_last_error(void);
/* Wait for `stream`, then report (and clear) any device-side error flag. */
int mk_sync_status(void *stream);

/* --- staging ---------------------------------------------------------- */
/* Per-pixel prologue. Replaces the per-pixel set-up inside
 * compute_scattering_cffi (Beam.py:716-746) and pixel_phasor (Beam.py:9241-9255). */
int mk_pixels_prepare(const mk_pixels *px, const mk_physics *phys, void *stream);

/* The scattering factor (f0 + f' + i f'') e^{-B s^2} sqrt(P_pol) of every
 * species at every pixel's own direction, into px->factor (n_species, n_pix,
 * 2) float32: once per (species, pixel), where the reference evaluates f0,
 * f'/f'' and the polarization factor per (atom, pixel) (Beam.py:770-806).
 * The split kernels read it when px->factor is set (spherical decay still per
 * tile and pixel); the caller admits it where the tile origins stay close to
 * the sample origin against the pixel distance (the direction to a tile then
 * differs from the pixel's by 2 (|o| + r) / R0 < 1e-6). n_frames > 1: each
 * pixel's incident direction and polarization from its frame in frames_dev
 * (mk_scan_plan's table, on the device); else phys->beam_dir, phys->pol_e.
 * remove_forward is refused (its Q < Q_cut test stays per tile and pixel). */
int mk_factor_table(const mk_pixels *px, const mk_species *sp, const mk_physics *phys,
                    int n_frames, const mk_frame_desc *frames_dev, void *stream);

/* Stage transform and incident amplitude per atom. Replaces the float32
 * `pos @ R.T + T` of interact_beam_gpu/cpu (Beam.py:6277-6280, 5896-5902)
 * and ein_bilinear_kernel / _ein_bilinear_cpu with tau = phi = 0
 * (Beam.py:2439-2578, 956-1045): E_in is E0 sampled bilinearly on the beam
 * grid, 0 outside it.
 *   pos_in:  device (n, 3) float32 [A] sample frame
 *   rot, trans: host (9) row-major float32 rotation and (3) translation [A]
 *   e0: device (grid_ny, grid_nz) complex64 beam map (NULL: amplitude 1)
 *   grid: host du, dv, uc, vc (Beam.py:228-231)
 *   pos_lab: device (n, 3) float64 [m] (float32 lab position / 1e10)
 *   amp: device (n, 2) float32 */
int mk_atoms_lab(int64_t n, const float *pos_in, const float *rot, const float *trans,
                 const float *e0, int grid_ny, int grid_nz, const double *grid,
                 double *pos_lab, float *amp, void *stream);

/* --- depth-dependent incident field (Beam.py:956-1045, 4963-5140,
 * 5583-5618, 7118-7283) ---------------------------------------------------
 * Column sums of the forward scattering factors on the beam grid (the
 * transmission map's input, _compute_beam_column_A_map_*): every atom inside
 * the grid deposits fwd[species] = (f0(0) + f', f'') with 3 x 3
 * triangular-shaped-cloud weights around its grid position (+x beam:
 * u = y, v = z). pos_lab: device (n, 3) float64 [m] from mk_atoms_lab;
 * fwd: device (n_species, 2) float32; grid: host du, dv, uc, vc [A];
 * sum_re, sum_im: device (grid_ny, grid_nz) float32, overwritten. */
int mk_beam_column_sums(int64_t n, const double *pos_lab, const int *species, const float *fwd,
                        int n_species, int grid_ny, int grid_nz, const double *grid,
                        float *sum_re, float *sum_im, void *stream);
/* Column sums -> tau = max(k beta, 0), phi = -k delta with
 * delta, beta = r_e lambda^2 / (2 pi du dv) x sums (float32 maps). */
int mk_beam_column_maps(int grid_ny, int grid_nz, const float *sum_re, const float *sum_im,
                        double wavelength_A, double du_A, double dv_A, float *tau, float *phi,
                        void *stream);
/* tau, phi in place through A = exp(-tau + i phi): tau = -log(|A| + 1e-20),
 * phi = arg A (the reference reads its maps back from the complex map). */
int mk_beam_column_wrap(int grid_ny, int grid_nz, float *tau, float *phi, void *stream);
/* Per-atom amplitude E0 exp(-f tau) exp(i f phi), E0, tau, phi sampled
 * bilinearly at the atom's grid position, f = clip((x - s_min) /
 * (s_max - s_min), 0, 1) its depth fraction along the +x beam; zero outside
 * the grid. Overwrites amp (n, 2) float32. */
int mk_atoms_ein_depth(int64_t n, const double *pos_lab, const float *e0, const float *tau,
                       const float *phi, int grid_ny, int grid_nz, const double *grid,
                       double s_min, double s_max, float *amp, void *stream);

/* Bytes of workspace mk_tiles_build needs for n atoms. */
size_t mk_tiles_workspace_size(int64_t n);
/* Species-partitioned space-filling order and tile build. Replaces
 * _partition, _morton_order_gpu, _chunk_origins_gpu and _stage
 * (Beam.py:9297-9319, 1204-1300, 9265-9294): atoms sorted by (species,
 * Hilbert index) -- a Hilbert curve instead of the reference's Z-order, so
 * no tile spans a Z-order jump -- then cut into tiles of `tiles->tile_atoms`
 * atoms whose origin is the FP64 bounding-box centre.
 *   pos: device (n, 3) float64 [m]; species: device (n) int32 in [0, S);
 *   amp: device (n, 2) float32; counts: host (S) atoms per species.
 *   tiles->n_tiles must equal sum_s ceil(counts[s] / tile_atoms). */
int mk_tiles_build(int64_t n, const double *pos, const int *species, const float *amp,
                   int n_species, const int64_t *counts, double k, mk_tiles *tiles,
                   void *workspace, size_t ws_bytes, void *stream);

/* --- sums ------------------------------------------------------------- */
/* Bytes of workspace the sums need (partial fields of `slices` slices). */
size_t mk_sum_workspace_size(int n_pix, int slices);

/* FP64 plain direct sum, term for term as compute_scattering_cffi
 * (Beam.py:748-808), added into (accumulate = 1) or written to `out`.
 *   pos: device (n, 3) float64 [m]; species: device (n) int32; amp: device (n, 2)
 *   out: device (2, n_pix) interleaved complex128 field (including r_e) */
int mk_kin_plain_f64(int64_t n, const double *pos, const int *species, const float *amp,
                     const mk_species *sp, const mk_physics *phys, const mk_pixels *px,
                     int slices, double *out, int accumulate, void *workspace,
                     size_t ws_bytes, void *stream);

/* Workspace bytes mk_kin_split_f32 needs for this launch (its work-item
 * counter and the partial fields of the slices it will choose). */
int mk_split_plan(const mk_tiles *tiles, const mk_pixels *px, const mk_launch *launch,
                  size_t *ws_bytes_out);

/* FP32 split-phase sum over tiles for one exposure (replaces the
 * `mosaic_fast` kernel and its dispatch, Beam.py:8114-8632, 9362-9496).
 * Same output convention as mk_kin_plain_f64. */
int mk_kin_split_f32(const mk_tiles *tiles, const mk_species *sp, const mk_physics *phys,
                     const mk_pixels *px, const mk_launch *launch, double *out,
                     int accumulate, void *workspace, size_t ws_bytes, void *stream);

/* Size of the fixed scratch array behind mk_kin_split_f32_noalloc: 32 MiB,
 * held in every GPU that loads this library until the process exits. */
#define MK_NOALLOC_SCRATCH_BYTES (32u << 20)

/* mk_kin_split_f32 for callers that cannot allocate device memory -- for
 * example a host application whose own memory pool owns all of the GPU's
 * memory and hands this library only the buffers it computes on, or a
 * service whose device memory is fixed when it starts. Same arguments and
 * result as mk_kin_split_f32, without the workspace: the scratch (a work
 * counter and the per-slice partial fields) lives in one fixed file-scope
 * device array of MK_NOALLOC_SCRATCH_BYTES, and the call allocates nothing
 * (no cudaMalloc, no cudaFree, no allocating library call). If the partial
 * fields of its usual slice count do not fit, it uses fewer slices; a
 * detector of more than (MK_NOALLOC_SCRATCH_BYTES - 256)/16 pixels (about
 * 2.1M) is rejected with MK_ENOMEM. The first call on a device (made with
 * that device current) looks up the array's device address and keeps it for
 * the life of the process, so make that first call before any stream
 * capture; after cudaDeviceReset of that device the kept address is stale
 * and this entry point must not be called again in the process. Every call
 * shares the array, and the call clears what must start at zero: calls that
 * may overlap on the GPU (other streams, other host threads) race and must
 * be serialised by the caller. No counterpart in the reference. */
int mk_kin_split_f32_noalloc(const mk_tiles *tiles, const mk_species *sp,
                             const mk_physics *phys, const mk_pixels *px,
                             const mk_launch *launch, double *out, int accumulate, void *stream);

/* --- batched scans ------------------------------------------------------ */
/* Plan a batched launch of n_frames frames (host only, no GPU work):
 * frame_pixels (n_frames) pixels per frame; frame_rows (n_frames) pixels per
 * detector row of each frame, or NULL (then no pixel quads); beam_dirs /
 * pol_es (n_frames, 3)
 * incident direction and polarization vector per frame in the sample frame.
 * Fills frames_out (host, n_frames) and the totals of work items and
 * partial-field entries. Copy frames_out to the device for mk_kin_scan_f32.
 * Replaces the per-step loop of experiment.scan_nD (Experiment.py:285-336),
 * which re-runs the whole exposure per step. */
int mk_scan_plan(int n_frames, const int *frame_pixels, const int *frame_rows,
                 const double *beam_dirs, const double *pol_es, const mk_tiles *tiles,
                 const mk_launch *launch,
                 mk_frame_desc *frames_out, long long *n_items, long long *n_partial);
size_t mk_scan_workspace_size(long long n_partial);

/* All frames of a scan in one persistent launch plus the FP64 reduction:
 * frames_dev, n_items and n_partial come from mk_scan_plan called with this
 * same launch (the pixel mode sets each frame's block count);
 * px holds the concatenated pixels of every frame (ny = total pixels,
 * nz = 1), each frame's prologue prepared with its own beam direction;
 * out (total pixels, 2) complex128 fields (r_e included);
 * intensity_sums (n_frames) sum of |A|^2 per frame, or NULL. Only kernel
 * launches and a memset: capturable in a CUDA graph when n_frames > 1. */
int mk_kin_scan_f32(const mk_tiles *tiles, const mk_species *sp, const mk_physics *phys,
                    const mk_pixels *px, int n_frames, const mk_frame_desc *frames_dev,
                    long long n_items, long long n_partial, const mk_launch *launch, double *out,
                    double *intensity_sums, void *workspace, size_t ws_bytes, void *stream);

/* --- free-space propagation ------------------------------------------- */
/* Replaces the pad / prop_mul_kernel / crop steps of
 * _angular_spectrum_propagate_gpu (Beam.py:7829-7943, 4747-4834); the FFTs
 * between them are the caller's (cuFFT). Arrays are interleaved complex64.
 * mk_prop_pad: (nz, ny) -> (nz2, ny2) placed at (z0, y0); mode 0 replicates
 * the edges, mode 1 fills with (cval_re, cval_im). */
int mk_prop_pad(const float *field, int ny, int nz, float *padded, int ny2, int nz2, int y0,
                int z0, int mode, float cval_re, float cval_im, void *stream);
/* In-place multiply of the (nz2, ny2) spectrum (FFT order, pitches dy, dz [m])
 * by the propagator over z [m] with the carrier (k_axis, k_perp_y, k_perp_z)
 * removed; k_axis = k for a forward beam. Phase formed in FP64. */
int mk_prop_mul(float *spectrum, int ny2, int nz2, double dy, double dz, double k, double z,
                double k_axis, double k_perp_y, double k_perp_z, void *stream);
/* The spectral step with the multiply fused into the transform: on the
 * (nz2, ny2) field already transformed along y (rows, FFT order), each
 * column is transformed along z in shared memory, multiplied by the same
 * propagator as mk_prop_mul (formed in FP32 as the reference's
 * prop_mul_kernel does, Beam.py:4763-4830, with the constant phases
 * z (k - k_axis) and -z k_axis reduced mod 2 pi in FP64) and transformed
 * back along z, unnormalised, in place. The caller's inverse row transform
 * then completes the inverse 2-D transform; the crop applies
 * 1 / (ny2 nz2). Replaces the column passes of the forward and inverse 2-D
 * FFTs and prop_mul_kernel's separate pass over the spectrum. nz2 a power
 * of two in [2, 8192], ny2 a power of two; workspace of
 * mk_prop_cols_workspace_size bytes (twiddle and wavenumber tables),
 * 16-byte aligned. */
size_t mk_prop_cols_workspace_size(int ny2, int nz2);
int mk_prop_cols(float *spectrum, int ny2, int nz2, double dy, double dz, double k, double z,
                 double k_axis, double k_perp_y, double k_perp_z, void *workspace, size_t ws_bytes,
                 void *stream);
/* Centre crop (nz, ny) at (z0, y0) of the inverse transform times `scale`,
 * fused with |A|^2: writes field (complex64) and/or intensity (float32). */
int mk_prop_crop_abs2(const float *grid, int ny2, int nz2, int y0, int z0, int ny, int nz,
                      float scale, float *field, float *intensity, void *stream);

/* --- tensor cores (tcgen05) --------------------------------------------- */
/* No counterpart in the reference: the self-check of the library's
 * tensor-core path. C (128 x N, float32, row-major) = A (128 x K) . B^T with
 * B (N x K), both row-major 16-bit (FP16, or BF16 when bf16 != 0), on one
 * tcgen05.mma tile accumulating in tensor memory: it exercises the operand
 * and instruction descriptors and the TMEM round trip the other tcgen05
 * kernels use. N a multiple of 16 in [16, 256], K a multiple of 16 in
 * [16, 128]; device pointers. */
int mk_tc_gemm(int N, int K, int bf16, const void *A, const void *B, float *C, void *stream);

/* --- scan surrogate (BF16 MLP) ------------------------------------------ */
/* No counterpart in the reference: the learned part of the scan path. BF16
 * operands, FP32 accumulation on the tensor cores (mma.sync m16n8k16).
 * C[M,N] (+)= A[M,K] B[K,N]: A(m,k) at A[m*sam + k*sak], B(k,n) at
 * B[k*sbk + n*sbn] (bf16); C float32 row stride ldc (or NULL); Cb bf16 copy
 * row stride ldcb (or NULL); flags: 1 accumulate into C, 2 add bias[n],
 * 4 ReLU. */
int mk_gemm_bf16(int M, int N, int K, const void *A, long long sam, long long sak, const void *B,
                 long long sbk, long long sbn, float *C, long long ldc, const float *bias,
                 int flags, void *Cb, long long ldcb, void *stream);
/* The same product on the Blackwell tensor cores (tcgen05.mma, FP32
 * accumulation in tensor memory), same operand conventions, with a fused
 * epilogue: v = A.B (+ bias[n]) (+ C[m, n] when flags & 1), ReLU (flags & 4),
 * then zero where relu_mask[m*ldm + n] <= 0 (relu_mask non-NULL: the
 * derivative of a ReLU layer whose outputs relu_mask holds), times
 * row_scale[m] (non-NULL), stored at row row_map[m] of C / Cb (non-NULL;
 * not with flags & 1). A CTA computes a 128 x 64 (N >= 2048: 128 x 128)
 * tile through three 64-deep shared-memory stages; long-K, few-tile
 * products (the weight gradients) split K over up to 8 CTAs that add into
 * a zeroed C. */
int mk_gemm_tc(int M, int N, int K, const void *A, long long sam, long long sak, const void *B,
               long long sbk, long long sbn, float *C, long long ldc, const float *bias, int flags,
               void *Cb, long long ldcb, const float *relu_mask, long long ldm,
               const float *row_scale, const long long *row_map, void *stream);
/* mk_gemm_tc over `groups` independent products of the same shape in one
 * launch (grid z = group): group q reads A + q*gs[0], B + q*gs[1], bias +
 * q*gs[4], relu_mask + q*gs[5] and writes C + q*gs[2], Cb + q*gs[3], with
 * gs = group_strides (6 element strides, host array; a stride of 0 shares
 * an input between groups). row_scale / row_map need groups == 1. */
int mk_gemm_tc_groups(int groups, const long long *group_strides, int M, int N, int K,
                      const void *A, long long sam, long long sak, const void *B, long long sbk,
                      long long sbn, float *C, long long ldc, const float *bias, int flags,
                      void *Cb, long long ldcb, const float *relu_mask, long long ldm,
                      const float *row_scale, const long long *row_map, void *stream);
/* Inputs of the network: (x, y) and sin/cos(2 pi f_j x), sin/cos(2 pi f_j y),
 * f_j = f0 ratio^j, j < n_freq, zero-padded to `width` bf16 columns. */
int mk_fourier_features(int n, const float *xy, int n_freq, float f0, float ratio, int width,
                        void *out, void *stream);
int mk_relu_backward(long long n, const float *grad, const float *pre, float *gout,
                     void *gout_bf16, void *stream);
/* db[n] = sum over rows m of g[m, n] (g row-major M x N); the _groups form
 * does `groups` of them at once: g + q*g_stride -> db + q*db_stride. */
int mk_bias_grad(int M, int N, const float *g, float *db, void *stream);
int mk_bias_grad_groups(int groups, int M, int N, const float *g, long long g_stride, float *db,
                        long long db_stride, void *stream);
/* MSE over n entries: grad = 2(y - t)/n (float and/or bf16), partial sums of
 * squares per 256-block in `partials` (ceil(n/256) doubles). */
int mk_mse(long long n, const float *y, const float *t, float *grad, void *grad_bf16,
           double *partials, void *stream);
/* The same with entry (i, j) of the row-major (n / n_col, n_col) arrays
 * weighted by col_w[j]: grad = 2 w (y - t)/n, partial sums of w (y - t)^2. */
int mk_mse_weighted(long long n, int n_col, const float *y, const float *t, const float *col_w,
                    float *grad, void *grad_bf16, double *partials, void *stream);
/* Adam step `step` (1-based) on FP32 master weights w, moments m, v; writes
 * the bf16 copy w_bf16 (or NULL). */
int mk_adam(long long n, float *w, const float *g, float *m, float *v, void *w_bf16, float lr,
            float beta1, float beta2, float eps, int step, float weight_decay, void *stream);
/* mk_adam with the step in device memory: step t = *step + 1 and learning
 * rate lr_sched[*step - step0], so that a captured training step replays
 * with advancing steps; mk_counter_add(step, 1) ends each captured step. */
int mk_adam_sched(long long n, float *w, const float *g, float *m, float *v, void *w_bf16,
                  const float *lr_sched, const int *step, int step0, float beta1, float beta2,
                  float eps, float weight_decay, void *stream);
int mk_counter_add(int *counter, int delta, void *stream);

/* --- diagnostics ------------------------------------------------------ */
/* Pipe-throughput microbenchmark (no counterpart in the reference): results
 * per clock per SM of kind 0 MUFU sine, 1 MUFU sine+cosine (two results per
 * call), 2 FRND (rintf), 3 FFMA, 4 packed FFMA2 (counted in FMAs), over
 * one wave of blocks; `iters` loop trips
 * of eight chains per thread. Synchronises `stream`. Workspace of
 * mk_probe_workspace_size() bytes (device). Gives the split kernel's roofline
 * denominator on the GPU at hand. */
size_t mk_probe_workspace_size(void);
int mk_probe_throughput(int kind, int iters, void *workspace, size_t ws_bytes,
                        double *ops_per_clk_per_sm, void *stream);
/* Launch a kernel whose bounded mbarrier wait is never satisfied: it gives
 * up after limit_ns (<= 1 s), records a timeout, and mk_sync_status() then
 * returns MK_ETIMEOUT. Exercises the error path of the tile-copy waits
 * without faulting or hanging the GPU. No counterpart in the reference. */
int mk_debug_wait_timeout(uint64_t limit_ns, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* MOSAIC_KIN_H */
