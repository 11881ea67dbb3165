// sofi_tti.cu -- instantiations and launchers of the TTI stress kernels.
#include "sofi_dispatch.cuh"
#include "sofi_kernels.cuh"
#include "sofi_launch.h"

namespace sofi {

void launch_tti_fused(const Geo &G, const Wave &W, const Model &M, int nd, bool visco, bool cpml, dim3 grd,
                      cudaStream_t st)
{
    const dim3 blk(BX, BY);
    if (visco && cpml) {
        DISPATCH_ND(nd, (launch_pdl(k_tti_fused<ND, true, true>, grd, blk, 0, st, G, W, M)));
    } else if (visco) {
        DISPATCH_ND(nd, (launch_pdl(k_tti_fused<ND, true, false>, grd, blk, 0, st, G, W, M)));
    } else if (cpml) {
        DISPATCH_ND(nd, (launch_pdl(k_tti_fused<ND, false, true>, grd, blk, 0, st, G, W, M)));
    } else {
        DISPATCH_ND(nd, (launch_pdl(k_tti_fused<ND, false, false>, grd, blk, 0, st, G, W, M)));
    }
}

// The map of k_tti_tiles. The interior rectangle: cells whose ring (one cell
// each side) lies in the interior region gx2 < i <= gx3, gy2 < j <= gy3 and in
// the grid; its first column i0 has i0 - 1 a multiple of 4, its width is a
// multiple of 4.
static TtiMap tti_map(const Geo &G)
{
    TtiMap T{};
    T.nsx = (G.nx + BX - 1) / BX, T.nsy = (G.ny + BY - 1) / BY;
    const int xhi = G.gx3 < G.nx ? G.gx3 : G.nx, yhi = G.gy3 < G.ny ? G.gy3 : G.ny;
    T.fi0 = ((G.gx2 + 4) / 4) * 4 + 1;  // the first i >= gx2 + 2 with i - 1 = 0 mod 4
    T.fi1 = T.fi0 + ((xhi - 1 - T.fi0 + 1) / 4) * 4 - 1;
    T.fj0 = G.gy2 + 2, T.fj1 = yhi - 1;
    if (T.fi1 < T.fi0 || T.fj1 < T.fj0) {  // no interior rectangle: every 32 x 8 tile is a frame tile
        T.fi0 = 1, T.fi1 = 0, T.fj0 = 1, T.fj1 = 0;
        T.sxa = 0, T.sxb = -1, T.sya = T.nsy, T.syb = T.nsy - 1;
        T.nframe = T.nsx * T.nsy;
        return T;
    }
    T.nfx = (T.fi1 - T.fi0 + T4X) / T4X, T.nfy = (T.fj1 - T.fj0 + T4Y) / T4Y;
    // 32 x 8 tiles wholly inside: 32 sx + 1 >= fi0 and 32 sx + 32 <= fi1 (rows likewise)
    T.sxa = (T.fi0 - 1 + BX - 1) / BX, T.sxb = T.fi1 / BX - 1;
    T.sya = (T.fj0 - 1 + BY - 1) / BY, T.syb = T.fj1 / BY - 1;
    if (T.sxb < T.sxa || T.syb < T.sya)
        T.sxa = 0, T.sxb = -1, T.sya = T.nsy, T.syb = T.nsy - 1;
    T.nframe = T.nsx * T.nsy - (T.sxb - T.sxa + 1) * (T.syb - T.sya + 1);
    return T;
}

void launch_tti_tiles(const Geo &G, const Wave &W, const Model &M, int nd, bool visco, bool cpml, cudaStream_t st)
{
    const TtiMap T = tti_map(G);
    const unsigned n = T.nframe + T.nfx * T.nfy;
    const dim3 grd = G.shot_fast ? dim3(n * G.nshots, 1, 1) : dim3(n, 1, G.nshots), blk(BX * BY);
    if (visco && cpml) {
        DISPATCH_ND(nd, (launch_pdl(k_tti_tiles<ND, true, true>, grd, blk, 0, st, G, W, M, T)));
    } else if (visco) {
        DISPATCH_ND(nd, (launch_pdl(k_tti_tiles<ND, true, false>, grd, blk, 0, st, G, W, M, T)));
    } else if (cpml) {
        DISPATCH_ND(nd, (launch_pdl(k_tti_tiles<ND, false, true>, grd, blk, 0, st, G, W, M, T)));
    } else {
        DISPATCH_ND(nd, (launch_pdl(k_tti_tiles<ND, false, false>, grd, blk, 0, st, G, W, M, T)));
    }
}

void launch_tti_split(const Geo &G, const Wave &W, const Model &M, int nd, bool visco, dim3 grd, cudaStream_t st)
{
    const dim3 blk(BX, BY);
    DISPATCH_ND(nd, (k_tti_deriv<ND><<<grd, blk, 0, st>>>(G, W, M)));
    if (visco)
        k_update_s_tti<true><<<grd, blk, 0, st>>>(G, W, M);
    else
        k_update_s_tti<false><<<grd, blk, 0, st>>>(G, W, M);
}

}  // namespace sofi
