// Split-phase kernel instances for 2x2 pixel quads with 4 pixels a thread
// (one quad; 64/128/256 threads, Fresnel/complex variants; no analyser) and
// the quad picker. The 8-pixel instances are in mk_split_quad8.cu, so the two
// halves compile in parallel.
#include "mk_split.cuh"

mk_split_fn mk_pick_quad8(int nt, bool fresnel, bool cplx);

mk_split_fn mk_pick_quad(int nt, int pix, bool fresnel, bool cplx)
{
    if (pix == 8) return mk_pick_quad8(nt, fresnel, cplx);
    if (pix != 4) return nullptr;
    switch (nt) {
    case 64: return mk_pick4<64, 4, 2, false>(fresnel, cplx);
    case 128: return mk_pick4<128, 4, 2, false>(fresnel, cplx);
    case 256: return mk_pick4<256, 4, 2, false>(fresnel, cplx);
    default: return nullptr;
    }
}
