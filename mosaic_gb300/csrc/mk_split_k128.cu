// Split-phase kernel instances for blocks of 128 threads (all pixel
// counts, Fresnel/complex/pair/analyser variants the picker allows).
#include "mk_split.cuh"

mk_split_fn mk_pick_nt128(int pix, bool fresnel, bool cplx, bool pair, bool ana)
{
    MK_PIX_CASES(128)
}
