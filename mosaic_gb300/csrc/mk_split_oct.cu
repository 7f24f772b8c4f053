// Split-phase kernel instances for 2x4 pixel octets (two 2x2 quads side by
// side sharing their half differences; 8 pixels a thread; 64/128/256
// threads, Fresnel/complex variants; no analyser).
#include "mk_split.cuh"

mk_split_fn mk_pick_oct(int nt, int pix, bool fresnel, bool cplx, bool ana)
{
    if (ana || pix != 8) return nullptr;
    switch (nt) {
    case 64: return mk_pick4<64, 8, 3, false>(fresnel, cplx);
    case 128: return mk_pick4<128, 8, 3, false>(fresnel, cplx);
    case 256: return mk_pick4<256, 8, 3, false>(fresnel, cplx);
    default: return nullptr;
    }
}
