// sofi_velocity.cu -- instantiations and launcher of the velocity kernels.
#include "sofi_dispatch.cuh"
#include "sofi_kernels.cuh"
#include "sofi_launch.h"

namespace sofi {

void launch_velocity(const Geo &G, const Wave &W, const Model &M, int nd, int vw, int vrows, bool narrow, bool acoustic,
                     dim3 gv, cudaStream_t st, const FwiDev *bwd)
{
    const dim3 blk(BX, BY);
    if (bwd) {  // a backward step of an FWI pass: 4, 2 or 1 cells per thread (vrows is 1 then)
        const FwiDev &F = *bwd;
        if (vw == 4)
            DISPATCH_ND(nd, (launch_pdl(k_update_vw_bwd<ND, 4>, gv, blk, 0, st, G, W, M, F)))
        else if (vw == 2)
            DISPATCH_ND(nd, (launch_pdl(k_update_vw_bwd<ND, 2>, gv, blk, 0, st, G, W, M, F)))
        else
            DISPATCH_ND(nd, (launch_pdl(k_update_vw_bwd<ND, 1>, gv, blk, 0, st, G, W, M, F)))
        return;
    }
    if (narrow && vw == 4 && narrow_v_applies(acoustic, W.fa_x != nullptr)) {
        DISPATCH_ND(nd, (launch_pdl(k_update_vw<ND, 4, true, false, 8>, gv, dim3(8, BX * BY / 8), 0, st, G, W, M)))
        return;
    }
    if (acoustic) {
        if (vw == 4)
            DISPATCH_ND(nd, (launch_pdl(k_update_vw<ND, 4, false>, gv, blk, 0, st, G, W, M)))
        else if (vw == 2)
            DISPATCH_ND(nd, (launch_pdl(k_update_vw<ND, 2, false>, gv, blk, 0, st, G, W, M)))
        else
            DISPATCH_ND(nd, (launch_pdl(k_update_vw<ND, 1, false>, gv, blk, 0, st, G, W, M)))
        return;
    }
    if (W.fa_x) {  // a step of an FWI forward run: 4, 2 or 1 cells per thread (vrows is 1 then)
        if (vw == 4)
            DISPATCH_ND(nd, (launch_pdl(k_update_vw<ND, 4, true, true>, gv, blk, 0, st, G, W, M)))
        else if (vw == 2)
            DISPATCH_ND(nd, (launch_pdl(k_update_vw<ND, 2, true, true>, gv, blk, 0, st, G, W, M)))
        else
            DISPATCH_ND(nd, (launch_pdl(k_update_vw<ND, 1, true, true>, gv, blk, 0, st, G, W, M)))
        return;
    }
    if (vw == 4)
        DISPATCH_ND(nd, (launch_pdl(k_update_vw<ND, 4>, gv, blk, 0, st, G, W, M)))
    else if (vw == 2)
        DISPATCH_ND(nd, (launch_pdl(k_update_vw<ND, 2>, gv, blk, 0, st, G, W, M)))
    else if (vrows == 2)
        DISPATCH_ND(nd, (launch_pdl(k_update_v<ND, 2>, gv, blk, 0, st, G, W, M)))
    else if (vrows == 4)
        DISPATCH_ND(nd, (launch_pdl(k_update_v<ND, 4>, gv, blk, 0, st, G, W, M)))
    else
        DISPATCH_ND(nd, (launch_pdl(k_update_v<ND, 1>, gv, blk, 0, st, G, W, M)))
}

}  // namespace sofi
