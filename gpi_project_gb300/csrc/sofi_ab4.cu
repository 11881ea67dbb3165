// sofi_ab4.cu -- launchers of the FDORDER_TIME = 4 kernels (sofi_ab4.cuh).
#include "sofi_ab4.cuh"
#include "sofi_dispatch.cuh"
#include "sofi_launch.h"

namespace sofi {

void launch_ab4_begin(const Geo &G, cudaStream_t st)
{
    k_ab4_begin<<<1, 1, 0, st>>>(G);
}

namespace {
// blocks of the four-cell kernels (the one-cell kernels get the caller's grid)
dim3 grid4(const Geo &G)
{
    const unsigned tx = (G.nx + 4 * BX - 1) / (4 * BX), ty = (G.ny + BY - 1) / BY;
    return G.shot_fast ? dim3(tx * G.nshots, ty, 1) : dim3(tx, ty, G.nshots);
}
}  // namespace

void launch_ab4_v(const Geo &G, const Wave &W, const Model &M, int nd, bool wide, dim3 grd, cudaStream_t st)
{
    const dim3 blk(BX, BY);
    if (wide)
        DISPATCH_ND(nd, (k_update_v_ab4w<ND><<<grid4(G), blk, 0, st>>>(G, W, M)))
    else
        DISPATCH_ND(nd, (k_update_v_ab4<ND><<<grd, blk, 0, st>>>(G, W, M)))
}

void launch_ab4_s(const Geo &G, const Wave &W, const Model &M, int nd, bool visco, bool wide, dim3 grd,
                  cudaStream_t st)
{
    const dim3 blk(BX, BY);
    if (wide && visco)
        DISPATCH_ND(nd, (k_update_s_ab4w<ND, true><<<grid4(G), blk, 0, st>>>(G, W, M)))
    else if (wide)
        DISPATCH_ND(nd, (k_update_s_ab4w<ND, false><<<grid4(G), blk, 0, st>>>(G, W, M)))
    else if (visco)
        DISPATCH_ND(nd, (k_update_s_ab4<ND, true><<<grd, blk, 0, st>>>(G, W, M)))
    else
        DISPATCH_ND(nd, (k_update_s_ab4<ND, false><<<grd, blk, 0, st>>>(G, W, M)))
}

}  // namespace sofi
