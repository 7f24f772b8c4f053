// Split-phase kernel instances for 4x4 pixel squares with 192-thread blocks
// (two per SM with 1024-atom tiles: 12 warps; its own translation unit so
// that the build compiles it in parallel with the 128-thread instances).
#include "mk_split.cuh"

mk_split_fn mk_pick_sq192(bool fresnel, bool cplx)
{
    return mk_pick4<192, 16, 4, false>(fresnel, cplx);
}
