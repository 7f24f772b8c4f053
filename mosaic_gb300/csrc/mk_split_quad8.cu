// Split-phase kernel instances for 2x2 pixel quads with 8 pixels a thread
// (two quads; 64/128/256 threads, Fresnel/complex variants; no analyser).
#include "mk_split.cuh"

mk_split_fn mk_pick_quad8(int nt, bool fresnel, bool cplx)
{
    switch (nt) {
    case 64: return mk_pick4<64, 8, 2, false>(fresnel, cplx);
    case 128: return mk_pick4<128, 8, 2, false>(fresnel, cplx);
    case 256: return mk_pick4<256, 8, 2, false>(fresnel, cplx);
    default: return nullptr;
    }
}
