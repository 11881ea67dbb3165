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
