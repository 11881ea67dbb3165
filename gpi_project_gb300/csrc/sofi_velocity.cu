// sofi_velocity.cu -- instantiations and launcher of the velocity kernels.
#include "sofi_dispatch.cuh"
#include "sofi_kernels.cuh"
#include "sofi_launch.h"
#include "sofi_vpipe.cuh"

#include <cudaTypedefs.h>

#include <mutex>

namespace sofi {

void launch_velocity(const Geo &G, const Wave &W, const Model &M, int nd, int vw, int vrows, bool narrow, bool acoustic,
                     dim3 gv, cudaStream_t st)
{
    const dim3 blk(BX, BY);
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
    if (vw == 4 && W.fa_x)  // a step of an FWI forward run
        DISPATCH_ND(nd, (launch_pdl(k_update_vw<ND, 4, true, true>, gv, blk, 0, st, G, W, M)))
    else if (vw == 4)
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

namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// 2-D map over the padded rows of all shots; box `bw` x VT_RB floats
bool encode_field(PFN_cuTensorMapEncodeTiled_v12000 fn, CUtensorMap *m, const float *base, const Geo &G, int bw)
{
    const cuuint64_t dims[2] = {(cuuint64_t)G.pitch, (cuuint64_t)G.nshots * (cuuint64_t)(G.ny + 2 * HY)};
    const cuuint64_t strides[1] = {(cuuint64_t)G.pitch * sizeof(float)};
    const cuuint32_t box[2] = {(cuuint32_t)bw, (cuuint32_t)VT_RB};
    const cuuint32_t estr[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int ND>
const char *plan_nd(const Geo &G, const Wave &W, int device, VtPlan *plan)
{
    using S = VtShape<ND>;
    PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
    if (!fn)
        return "cuTensorMapEncodeTiled is not available";
    // the rows of all shots must fit the map's 32-bit coordinates
    if ((long long)G.nshots * (G.ny + 2 * HY) >= (1LL << 31))
        return "too many rows for a tensor map";
    if (!encode_field(fn, &plan->xx, W.sxx, G, S::SW) || !encode_field(fn, &plan->xy, W.sxy, G, S::SW) ||
        !encode_field(fn, &plan->yy, W.syy, G, VT_TW))
        return "tensor map encoding failed";
    static std::mutex mu;
    static int per_sm[7] = {0, 0, 0, 0, 0, 0, 0};
    {
        std::lock_guard<std::mutex> lk(mu);
        if (!per_sm[ND]) {
            // the largest shared-memory carveout, so that the resident blocks the
            // occupancy query counts are the ones the launch gets
            if (cudaFuncSetAttribute(k_update_vt<ND>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM) !=
                    cudaSuccess ||
                cudaFuncSetAttribute(k_update_vt<ND>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess ||
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm[ND], k_update_vt<ND>, VT_THREADS, S::SMEM) !=
                    cudaSuccess)
                per_sm[ND] = 0;
        }
        if (per_sm[ND] <= 0) {
            cudaGetLastError();
            return "no resident block of the velocity pipeline fits an SM";
        }
    }
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms <= 0)
        return "multiprocessor count unavailable";
    const int strips = (G.nx + VT_TW - 1) / VT_TW;
    const int nck = (G.ny + VT_RB - 1) / VT_RB;
    const long long cols = (long long)strips * G.nshots;
    long long segs = (long long)per_sm[ND] * sms / cols;  // one wave of resident blocks
    segs = segs < 1 ? 1 : (segs > nck ? nck : segs);
    plan->strips = strips;
    plan->segs = (int)segs;
    return nullptr;
}

}  // namespace

const char *plan_velocity_pipeline(const Geo &G, const Wave &W, int nd, int device, VtPlan *plan)
{
    plan->segs = 0;
    const char *msg = "unsupported FD order";
    DISPATCH_ND(nd, (msg = plan_nd<ND>(G, W, device, plan)));
    if (msg)
        plan->segs = 0;
    return msg;
}

void launch_velocity_pipeline(const Geo &G, const Wave &W, const Model &M, int nd, const VtPlan &p,
                              cudaStream_t st)
{
    const unsigned S = (unsigned)G.nshots;
    const dim3 grid = G.shot_fast ? dim3(p.strips * S, p.segs, 1) : dim3(p.strips, p.segs, S);
    DISPATCH_ND(nd, (k_update_vt<ND><<<grid, VT_THREADS, VtShape<ND>::SMEM, st>>>(G, W, M, p.xx, p.xy, p.yy)));
}

}  // namespace sofi
