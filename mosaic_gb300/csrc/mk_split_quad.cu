// Split-phase kernel instances for 2x2 pixel quads with 4 pixels a thread
// (one quad; 64/128/256 threads, Fresnel/complex variants) and the quad
// picker. The 8-pixel instances are in mk_split_quad8.cu and the analyser
// ones in mk_split_quad_ana.cu, so the three compile in parallel.
#include "mk_split.cuh"

mk_split_fn mk_pick_quad8(int nt, bool fresnel, bool cplx);
mk_split_fn mk_pick_quad_ana(int nt, int pix, bool fresnel, bool cplx);

mk_split_fn mk_pick_quad(int nt, int pix, bool fresnel, bool cplx, bool ana)
{
    if (ana) return mk_pick_quad_ana(nt, pix, fresnel, cplx);
    if (pix == 8) return mk_pick_quad8(nt, fresnel, cplx);
    if (pix != 4) return nullptr;
    switch (nt) {
    case 64: return mk_pick4<64, 4, 2, false>(fresnel, cplx);
    case 128: return mk_pick4<128, 4, 2, false>(fresnel, cplx);
    case 256: return mk_pick4<256, 4, 2, false>(fresnel, cplx);
    default: return nullptr;
    }
}
