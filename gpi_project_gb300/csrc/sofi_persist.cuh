// sofi_persist.cuh -- a chunk of time steps as one persistent kernel.
//
// On small grids a step's kernels run for a few microseconds each and the
// launches between them dominate. k_persist runs nsteps whole steps of an
// ISO / VTI / acoustic medium in one cooperative launch: per step the phases
//   force sources -> velocity update -> stress update -> per-column post
// (sources, free surface, NaN probe, sampling) are separated by a grid-wide
// barrier. Each phase walks the tiles of the plain launch's grid (tile t goes
// to block t mod gridDim.x) and runs the plain kernels' bodies on them
// (vw_tile, sw_tile / sac_tile, post_column, force_shot), so the arithmetic is
// that of the plain kernels with four cells per thread.
//
// Fields written in one phase and read by another (velocities, stresses) are
// loaded with ld.global.cg (L2, coherent) in the stencil bodies; the barrier
// orders every phase's writes before the next phase's reads (a fence on both
// sides of the arrival, as a grid-wide synchronisation does).
//
// The barrier is an arrival count and a generation word in device memory. A
// block that waits longer than kWaitNs sets bit 8 of G.fault and the kernel
// returns; every other block then gives up at its next barrier the same way.
// A cooperative launch guarantees that all blocks are resident, so the wait
// ends in a correct program.
#pragma once
#include "sofi_dispatch.cuh"
#include "sofi_kernels.cuh"

namespace sofi {

constexpr unsigned long long kBarrierWaitNs = 2000000000ull;

__device__ __forceinline__ unsigned long long persist_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Grid-wide barrier; false when the wait gave up (the caller returns).
__device__ __forceinline__ bool grid_barrier(const Geo &G, unsigned *bar, unsigned &gen)
{
    __shared__ int ok_s;
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        int ok = 1;
        const unsigned g = gen;
        const unsigned nb = gridDim.x * gridDim.y * gridDim.z;
        __threadfence();
        if (atomicAdd(&bar[0], 1u) == nb - 1) {
            atomicExch(&bar[0], 0u);
            __threadfence();
            atomicExch(&bar[1], g + 1);
        } else {
            const unsigned long long t0 = persist_ns();
            while (ld_acquire_u32(&bar[1]) == g)
                if (persist_ns() - t0 > kBarrierWaitNs) {
                    ok = 0;
                    if (G.fault)
                        atomicOr(G.fault, 8);
                    break;
                }
        }
        __threadfence();
        ok_s = ok;
    }
    __syncthreads();
    gen++;
    return ok_s != 0;
}

__device__ __forceinline__ uint3 tile_of(unsigned t, const unsigned *g)
{
    return make_uint3(t % g[0], (t / g[0]) % g[1], t / (g[0] * g[1]));
}

template <int ND, int KIND, bool VISCO, int LT>
__global__ void __launch_bounds__(BX *BY, 2) k_persist(Geo G, Wave W, Model M, Acq A, PersistArgs P)
{
    constexpr bool SXY = KIND != AC;
    const unsigned nb = gridDim.x;
    const int tid = threadIdx.y * BX + threadIdx.x;
    unsigned gen = *reinterpret_cast<volatile unsigned *>(&P.bar[1]);
    const unsigned nv = P.vg[0] * P.vg[1] * P.vg[2], ns = P.sg[0] * P.sg[1] * P.sg[2];
    const long long ncol = (long long)G.nx * G.nshots;
    for (int it = 0; it < P.nsteps; it++) {
        if (P.has_force) {
            for (int s = blockIdx.x * BX * BY + tid; s < G.nshots; s += nb * BX * BY)
                force_shot(G, W, M, A, s);
            if (!grid_barrier(G, P.bar, gen))
                return;
        }
        for (unsigned t = blockIdx.x; t < nv; t += nb)
            vw_tile<ND, 4, SXY, true>(G, W, M, tile_of(t, P.vg));
        if (!grid_barrier(G, P.bar, gen))
            return;
        for (unsigned t = blockIdx.x; t < ns; t += nb) {
            if (KIND == AC)
                sac_tile<ND, 4, true>(G, W, M, tile_of(t, P.sg));
            else
                sw_tile<ND, KIND, VISCO, LT, 4, true>(G, W, M, tile_of(t, P.sg));
        }
        if (!grid_barrier(G, P.bar, gen))
            return;
        for (long long q = (long long)blockIdx.x * BX * BY + tid; q < ncol; q += (long long)nb * BX * BY)
            post_column<ND, VISCO, false>(G, W, M, A, (int)(q % G.nx) + 1, (int)(q / G.nx));
        if (!grid_barrier(G, P.bar, gen))
            return;
    }
}

// Blocks of k_persist<ND, KIND, VISCO, L> that fit the GPU at once (0: none).
template <int KIND, bool VISCO>
int persist_capacity_kv(int nd, int L, int device)
{
    int per_sm = 0, sms = 0;
    cudaError_t e = cudaErrorInvalidValue;
#define SOFI_PERSIST_OCC(LT_)                                                                                    \
    DISPATCH_ND(nd, (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_persist<ND, KIND, VISCO, LT_>, \
                                                                       BX * BY, 0)))
    if (!VISCO) {
        SOFI_PERSIST_OCC(0);
    } else if (L == 1) {
        SOFI_PERSIST_OCC(1);
    } else if (L == 2) {
        SOFI_PERSIST_OCC(2);
    } else if (L == 3) {
        SOFI_PERSIST_OCC(3);
    } else {
        SOFI_PERSIST_OCC(0);
    }
#undef SOFI_PERSIST_OCC
    if (e != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return per_sm * sms;
}

template <int KIND, bool VISCO>
cudaError_t launch_persist_kv(const Geo &G, const Wave &W, const Model &M, const Acq &A, int nd,
                              const PersistArgs &P, int blocks, cudaStream_t st)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(BX, BY);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = cudaErrorInvalidValue;
    const int L = VISCO ? G.L : 0;
#define SOFI_PERSIST_LAUNCH(LT_) \
    DISPATCH_ND(nd, (e = cudaLaunchKernelEx(&cfg, k_persist<ND, KIND, VISCO, LT_>, G, W, M, A, P)))
    if (!VISCO) {
        SOFI_PERSIST_LAUNCH(0);
    } else if (L == 1) {
        SOFI_PERSIST_LAUNCH(1);
    } else if (L == 2) {
        SOFI_PERSIST_LAUNCH(2);
    } else if (L == 3) {
        SOFI_PERSIST_LAUNCH(3);
    } else {
        SOFI_PERSIST_LAUNCH(0);
    }
#undef SOFI_PERSIST_LAUNCH
    return e;
}

}  // namespace sofi
