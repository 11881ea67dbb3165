// sofi_stress_ac.cu -- acoustic stress kernels (one pressure field).
#include "sofi_dispatch.cuh"
#include "sofi_kernels.cuh"
#include "sofi_launch.h"

namespace sofi {

void launch_stress_ac(const Geo &G, const Wave &W, const Model &M, int nd, int sw, dim3 grd, cudaStream_t st)
{
    const dim3 blk(BX, BY);
    if (sw == 4)
        DISPATCH_ND(nd, (launch_pdl(k_update_s_ac<ND, 4>, grd, blk, 0, st, G, W, M)))
    else if (sw == 2)
        DISPATCH_ND(nd, (launch_pdl(k_update_s_ac<ND, 2>, grd, blk, 0, st, G, W, M)))
    else
        DISPATCH_ND(nd, (launch_pdl(k_update_s_ac<ND, 1>, grd, blk, 0, st, G, W, M)))
}

}  // namespace sofi
