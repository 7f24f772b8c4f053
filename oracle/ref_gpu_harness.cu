// Launcher for the reference's GPU general kernel -- TEST INFRASTRUCTURE ONLY.
//
// Compiles the kernel source that oracle/ref_build.py extracts, unchanged,
// from the reference's Beam.py (beam.build_interaction_kernel) into
// oracle/_ref/ref_general.cu, and launches it the way the reference's
// interact_beam_gpu does on its general path (Beam.py:6211-6213,
// 6327-6366): 32 x 16 pixel blocks over the detector, a single global
// origin (apply_origin = 0), one beam channel with g = 0, the field
// accumulated in place. Nothing in the library links this; it is the
// comparator "the reference's own kernel on this GPU" and the analyser's
// pin to the reference.
#include <cuda_runtime.h>

// The kernel names its unroll factor in `#pragma unroll UNROLL_ATOMS`; NVRTC
// takes that macro, nvcc does not expand macros inside the pragma. Defining
// the name as itself keeps the source's own default out, and the constant
// below is what the pragma then reads (the reference's value, 4).
#define UNROLL_ATOMS UNROLL_ATOMS
constexpr int UNROLL_ATOMS = 4;

#include "_ref/ref_general.cu"

// All pointers are device pointers (float32 metres, complex64 interleaved).
// Returns a cudaError_t value (0 on success).
extern "C" int mkref_general(int n_atoms, const float *kx, const float *ky, const float *kz,
                             const float *px, const float *py, const float *pz,
                             const float2 *amp, const float2 *anom, const float *f0_params,
                             const float *f0_zero, const float *x, const float *y, const float *z,
                             float2 *field, int ny, int nz, int remove_forward,
                             int apply_polarization, int spherical_decay, float pol_perp_rate,
                             int analyser_kind, float cx, float cy, float cz, float accept_rad,
                             float darwin_hw_rad, const float *zeros3, void *stream)
{
    if (n_atoms <= 0 || ny <= 0 || nz <= 0) return (int)cudaErrorInvalidValue;
    const dim3 block(32, 16);
    const dim3 grid((ny + block.x - 1) / block.x, (nz + block.y - 1) / block.y);
    interaction_kernal<<<grid, block, 0, (cudaStream_t)stream>>>(
        n_atoms, kx, ky, kz, px, py, pz, amp, anom, f0_params, f0_zero, x, y, z, field, ny, nz,
        remove_forward, apply_polarization, spherical_decay, pol_perp_rate,
        analyser_kind != 0 ? 1 : 0, analyser_kind, cx, cy, cz, accept_rad, darwin_hw_rad, zeros3,
        0, zeros3);
    return (int)cudaGetLastError();
}
