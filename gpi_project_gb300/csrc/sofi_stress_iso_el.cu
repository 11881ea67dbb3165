// sofi_stress_iso_el.cu -- stress kernels of ISO media, VISCO = false.
#include "sofi_stress.cuh"

namespace sofi {
void launch_stress_bwd(const Geo &G, const Wave &W, const Model &M, const FwiDev &F, int nd, int sw, dim3 grd,
                       cudaStream_t st, const Acq *post)
{
    const dim3 blk(BX, BY);
    if (post)  // one cell per thread with k_post's work
        DISPATCH_ND(nd, (launch_pdl(k_update_s_post_fwi<ND, true>, grd, blk, 0, st, G, W, M, *post, F)))
    else if (sw == 4)
        DISPATCH_ND(nd, (launch_pdl(k_update_sw_bwd<ND, 4>, grd, blk, 0, st, G, W, M, F)))
    else if (sw == 2)
        DISPATCH_ND(nd, (launch_pdl(k_update_sw_bwd<ND, 2>, grd, blk, 0, st, G, W, M, F)))
    else
        DISPATCH_ND(nd, (launch_pdl(k_update_sw_bwd<ND, 1>, grd, blk, 0, st, G, W, M, F)))
}

template void launch_stress_kv<ISO, false>(const Geo &, const Wave &, const Model &, int, int, bool, dim3,
                                        cudaStream_t, const Acq *);
}
