// sofi_ab4.cu -- launchers of the FDORDER_TIME = 4 kernels (sofi_ab4.cuh).
#include "sofi_ab4.cuh"
#include "sofi_dispatch.cuh"
#include "sofi_launch.h"

namespace sofi {

void launch_ab4_begin(const Geo &G, cudaStream_t st)
{
    k_ab4_begin<<<1, 1, 0, st>>>(G);
}

void launch_ab4_v(const Geo &G, const Wave &W, const Model &M, int nd, dim3 grd, cudaStream_t st)
{
    const dim3 blk(BX, BY);
    DISPATCH_ND(nd, (k_update_v_ab4<ND><<<grd, blk, 0, st>>>(G, W, M)))
}

void launch_ab4_s(const Geo &G, const Wave &W, const Model &M, int nd, bool visco, dim3 grd, cudaStream_t st)
{
    const dim3 blk(BX, BY);
    if (visco)
        DISPATCH_ND(nd, (k_update_s_ab4<ND, true><<<grd, blk, 0, st>>>(G, W, M)))
    else
        DISPATCH_ND(nd, (k_update_s_ab4<ND, false><<<grd, blk, 0, st>>>(G, W, M)))
}

}  // namespace sofi
