// Split-phase kernel instances for 4x4 pixel squares (four 2x2 quads
// sharing their half differences; 16 pixels a thread, Fresnel/complex
// variants; no analyser). The square loop is held to 12 warps per SM (~168
// registers a thread): three 128-thread blocks where their shared memory
// fits (tiles of up to 1024 atoms with the compact Kahan state), else two;
// 192-thread blocks (two per SM) are in mk_split_sq192.cu.
#include "mk_split.cuh"

mk_split_fn mk_pick_sq192(bool fresnel, bool cplx);

mk_split_fn mk_pick_sq(int nt, int pix, bool fresnel, bool cplx, bool ana)
{
    if (ana || pix != 16) return nullptr;
    if (nt == 128) return mk_pick4<128, 16, 4, false>(fresnel, cplx);
    if (nt == 192) return mk_pick_sq192(fresnel, cplx);
    return nullptr;
}
