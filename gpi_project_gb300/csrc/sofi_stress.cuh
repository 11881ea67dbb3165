// sofi_stress.cuh -- launcher template of the ISO / VTI stress kernels; each
// (kind, visco) pair is instantiated in its own translation unit.
#pragma once
#include "sofi_dispatch.cuh"
#include "sofi_kernels.cuh"
#include "sofi_launch.h"

namespace sofi {

template <int KIND, bool VISCO, int VW>
void stress_w(const Geo &G, const Wave &W, const Model &M, int nd, bool narrow, dim3 grd, cudaStream_t st)
{
    const dim3 blk(BX, BY);
    [[maybe_unused]] const int L = VISCO ? G.L : 0;
    if constexpr (VW == 4)
        if (narrow && narrow_s_applies(VISCO, L, W.fa_x != nullptr)) {  // 8 x 32 threads, 32 x 32 cells
            const dim3 nb(8, BX * BY / 8);
            if constexpr (!VISCO) {
                DISPATCH_ND(nd, (launch_pdl(k_update_sw<ND, KIND, false, 0, 4, false, 8>, grd, nb, 0, st, G, W, M)))
            } else {
                if (L == 1)
                    DISPATCH_ND(nd, (launch_pdl(k_update_sw<ND, KIND, true, 1, 4, false, 8>, grd, nb, 0, st, G, W, M)))
                else if (L == 2)
                    DISPATCH_ND(nd, (launch_pdl(k_update_sw<ND, KIND, true, 2, 4, false, 8>, grd, nb, 0, st, G, W, M)))
                else
                    DISPATCH_ND(nd, (launch_pdl(k_update_sw<ND, KIND, true, 3, 4, false, 8>, grd, nb, 0, st, G, W, M)))
            }
            return;
        }
    if constexpr (KIND == ISO && !VISCO)
        if (W.fa_x) {  // a step of an FWI forward run
            DISPATCH_ND(nd, (launch_pdl(k_update_sw<ND, ISO, false, 0, VW, true>, grd, blk, 0, st, G, W, M)))
            return;
        }
    if constexpr (!VISCO) {
        DISPATCH_ND(nd, (launch_pdl(k_update_sw<ND, KIND, false, 0, VW>, grd, blk, 0, st, G, W, M)))
    } else {
        if (L == 1)
            DISPATCH_ND(nd, (launch_pdl(k_update_sw<ND, KIND, true, 1, VW>, grd, blk, 0, st, G, W, M)))
        else if (L == 2)
            DISPATCH_ND(nd, (launch_pdl(k_update_sw<ND, KIND, true, 2, VW>, grd, blk, 0, st, G, W, M)))
        else if (L == 3)
            DISPATCH_ND(nd, (launch_pdl(k_update_sw<ND, KIND, true, 3, VW>, grd, blk, 0, st, G, W, M)))
        else
            DISPATCH_ND(nd, (launch_pdl(k_update_sw<ND, KIND, true, 0, VW>, grd, blk, 0, st, G, W, M)))
    }
}

template <int KIND, bool VISCO>
void launch_stress_kv(const Geo &G, const Wave &W, const Model &M, int nd, int sw, bool narrow, dim3 grd,
                      cudaStream_t st, const Acq *post)
{
    if (sw == 4)
        return stress_w<KIND, VISCO, 4>(G, W, M, nd, narrow, grd, st);
    if (sw == 2)
        return stress_w<KIND, VISCO, 2>(G, W, M, nd, false, grd, st);
    const dim3 blk(BX, BY);
    [[maybe_unused]] const int L = VISCO ? G.L : 0;
    if constexpr (KIND == ISO && !VISCO)
        if (W.fa_x) {  // a step of an FWI forward run, one cell per thread
            if (post)  // with k_post's work (the FwiDev argument is not read)
                DISPATCH_ND(nd, (launch_pdl(k_update_s_post_fwi<ND, false>, grd, blk, 0, st, G, W, M, *post,
                                            FwiDev{})))
            else
                DISPATCH_ND(nd, (launch_pdl(k_update_sw<ND, ISO, false, 0, 1, true>, grd, blk, 0, st, G, W, M)))
            return;
        }
    if (post) {  // one cell per thread with k_post's work (k_update_s_post)
        const Acq &A = *post;
        if constexpr (!VISCO) {
            DISPATCH_ND(nd, (launch_pdl(k_update_s_post<ND, KIND, false, 0>, grd, blk, 0, st, G, W, M, A)))
        } else {
            if (L == 1)
                DISPATCH_ND(nd, (launch_pdl(k_update_s_post<ND, KIND, true, 1>, grd, blk, 0, st, G, W, M, A)))
            else if (L == 2)
                DISPATCH_ND(nd, (launch_pdl(k_update_s_post<ND, KIND, true, 2>, grd, blk, 0, st, G, W, M, A)))
            else if (L == 3)
                DISPATCH_ND(nd, (launch_pdl(k_update_s_post<ND, KIND, true, 3>, grd, blk, 0, st, G, W, M, A)))
            else
                DISPATCH_ND(nd, (launch_pdl(k_update_s_post<ND, KIND, true, 0>, grd, blk, 0, st, G, W, M, A)))
        }
        return;
    }
    if constexpr (!VISCO) {
        DISPATCH_ND(nd, (launch_pdl(k_update_s<ND, KIND, false, 0>, grd, blk, 0, st, G, W, M)))
    } else {
        if (L == 1)
            DISPATCH_ND(nd, (launch_pdl(k_update_s<ND, KIND, true, 1>, grd, blk, 0, st, G, W, M)))
        else if (L == 2)
            DISPATCH_ND(nd, (launch_pdl(k_update_s<ND, KIND, true, 2>, grd, blk, 0, st, G, W, M)))
        else if (L == 3)
            DISPATCH_ND(nd, (launch_pdl(k_update_s<ND, KIND, true, 3>, grd, blk, 0, st, G, W, M)))
        else
            DISPATCH_ND(nd, (launch_pdl(k_update_s<ND, KIND, true, 0>, grd, blk, 0, st, G, W, M)))
    }
}

}  // namespace sofi
