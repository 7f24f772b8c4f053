// Split-phase kernel instances for 2x2 pixel quads with the analyser (128 or
// 256 threads, 4 or 8 pixels a thread, Fresnel/complex variants).
#include "mk_split.cuh"

template <int NT>
static mk_split_fn mk_pick_quad_ana_nt(int pix, bool fresnel, bool cplx)
{
    switch (pix) {
    case 4: return mk_pick4<NT, 4, 2, true>(fresnel, cplx);
    case 8: return mk_pick4<NT, 8, 2, true>(fresnel, cplx);
    default: return nullptr;
    }
}

mk_split_fn mk_pick_quad_ana(int nt, int pix, bool fresnel, bool cplx)
{
    switch (nt) {
    case 128: return mk_pick_quad_ana_nt<128>(pix, fresnel, cplx);
    case 256: return mk_pick_quad_ana_nt<256>(pix, fresnel, cplx);
    default: return nullptr;
    }
}
