// sofi_vpipe.cuh -- the velocity update (update_v_interior.c / update_v_PML.c /
// update_v_abs.c with wavefield_update_v.c) as a TMA-fed pipeline marching
// down column strips.
//
// Each block owns a strip of 128 columns (32 threads x 4 cells) over a segment
// of rows and walks it in chunks of 8 rows, one warp per row. A producer warp
// copies the chunk's sxx / sxy / syy tiles (x halo 4K columns; K = ceil(ND/4))
// into a ring of shared-memory stages with cp.async.bulk.tensor, each stage
// guarded by a full and an empty mbarrier. The y stencils of chunk k read rows
// of chunks k-1, k and k+1 (ND <= 8 rows), so every stress row leaves DRAM
// once per strip and up to three chunks are in flight ahead of the one being
// computed. vx, vy, rip and rjp are read with plain 16-byte loads one chunk
// ahead. The per-cell arithmetic is k_update_vw<ND, 4>'s, term by term.
//
// Index rules. Tensor maps are 2-D over the padded fields of all shots
// (width pitch, height nshots * (NY + 16)); the tile's first column
// i0 - 1 + HX - 4K is a multiple of 4, so every copy starts on a 16-byte
// boundary, and the box is 8 rows high with a width of 136 / 144 / 128 floats.
// A copy that reaches past the tensor is filled with zeros by the hardware;
// rows past NY + ND and columns past NX + ND only feed cells that are never
// stored. The pre-roll chunk above row 1 reads the ghost rows 0 .. 7.
//
// Waits. Every mbarrier wait gives up after kWaitNs of global time, sets a bit
// of G.fault (1 consumer, 2 producer, 4 producer drain) and leaves the loop;
// the producer then waits (bounded again) for the copies it issued before it
// exits, so no copy is in flight into a block that has ended. The host reads
// G.fault with the status words after a run.
#pragma once
#include <cuda.h>

#include "sofi_kernels.cuh"

namespace sofi {

constexpr int VT_RB = 8;                 // rows per chunk, one consumer warp each
constexpr int VT_NS = 6;                 // stages in the ring
constexpr int VT_TW = BX * 4;            // columns per strip
constexpr int VT_THREADS = (VT_RB + 1) * 32;
constexpr unsigned long long kWaitNs = 2000000000ull;

template <int ND>
struct VtShape {
    static constexpr int K = (ND + 3) / 4, HXs = 4 * K, SW = VT_TW + 2 * HXs;
    static constexpr int XX = 0, XY = VT_RB * SW, YY = 2 * VT_RB * SW;  // float offsets in a stage
    static constexpr int STAGE = 2 * VT_RB * SW + VT_RB * VT_TW;       // floats per stage
    static constexpr unsigned BYTES = STAGE * 4;
    static constexpr size_t SMEM = (size_t)VT_NS * STAGE * 4 + 128;   // + room to align the ring to 128 B
    static_assert((XY * 4) % 128 == 0 && (YY * 4) % 128 == 0 && BYTES % 128 == 0, "stage alignment");
};

__device__ __forceinline__ unsigned smem_u32(const void *p)
{
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(unsigned long long *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n"
        " .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Wait for the phase of the given parity to complete; false after kWaitNs.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity)
{
    if (mbar_try_wait(bar, parity))
        return true;
    const unsigned long long t0 = global_ns();
    while (!mbar_try_wait(bar, parity))
        if (global_ns() - t0 > kWaitNs)
            return false;
    return true;
}

__device__ __forceinline__ void tma_load_2d(float *dst, const CUtensorMap *map, unsigned long long *bar, int x,
                                            int y)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::
            "r"(smem_u32(dst)),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}

// Row r (-VT_RB <= r < 2 VT_RB, counted from the first row of chunk k) of a
// staged field: rows of chunks k-1, k, k+1 sit in stages prev, cur, next.
__device__ __forceinline__ const float *vt_row(const float *prev, const float *cur, const float *next, int off,
                                               int rw, int r)
{
    const float *b = r < 0 ? prev : (r >= VT_RB ? next : cur);
    return b + off + ((r + VT_RB) & (VT_RB - 1)) * rw;
}

template <int ND>
__global__ void __launch_bounds__(VT_THREADS, 2)
    k_update_vt(Geo G, Wave W, Model M, const __grid_constant__ CUtensorMap tm_xx,
                const __grid_constant__ CUtensorMap tm_xy, const __grid_constant__ CUtensorMap tm_yy)
{
    using S = VtShape<ND>;
    constexpr int K = S::K;
    __shared__ __align__(8) unsigned long long full[VT_NS], empty[VT_NS];
    extern __shared__ __align__(16) float vt_dyn[];
    float *ring = vt_dyn + ((128u - (smem_u32(vt_dyn) & 127u)) & 127u) / 4;
    int bx, s;
    block_xs(G, bx, s);
    if (G.step_ctr && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0)
        *G.step_ctr += 1;
    const int nck = (G.ny + VT_RB - 1) / VT_RB;  // chunks of the strip
    const int per = (nck + gridDim.y - 1) / gridDim.y;
    const int c0 = blockIdx.y * per, c1 = min(c0 + per, nck);
    if (c0 >= c1)
        return;
    const int nload = c1 - c0 + 2;  // chunks c0 - 1 .. c1: the segment and one chunk on either side
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int k = 0; k < VT_NS; k++) {
            mbar_init(&full[k], 1);
            mbar_init(&empty[k], VT_RB);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const int i0 = bx * VT_TW + 1;
    const int cx0 = i0 - 1 + HX - S::HXs;  // first staged column, a multiple of 4
    if (warp == VT_RB) {
        if (lane == 0) {
            const int srow = s * (G.ny + 2 * HY);
            int err = 0, k = 0;
            for (; k < nload; k++) {
                const int st = k % VT_NS;
                if (k >= VT_NS && !mbar_wait(&empty[st], ((k / VT_NS) - 1) & 1)) {
                    err = 2;
                    break;
                }
                float *b = ring + st * S::STAGE;
                const int y = srow + (c0 - 1 + k) * VT_RB + HY;  // padded row of the chunk's first row
                mbar_expect_tx(&full[st], S::BYTES);
                tma_load_2d(b + S::XX, &tm_xx, &full[st], cx0, y);
                tma_load_2d(b + S::XY, &tm_xy, &full[st], cx0, y);
                tma_load_2d(b + S::YY, &tm_yy, &full[st], cx0 + S::HXs, y);
            }
            // every copy issued has landed before this thread, and so the block, ends
            for (int q = k > VT_NS ? k - VT_NS : 0; q < k; q++)
                if (!mbar_wait(&full[q % VT_NS], (q / VT_NS) & 1))
                    err |= 4;
            if (err && G.fault)
                atomicOr(G.fault, err);
        }
        return;
    }
    const int w = warp, tx = lane;
    const int i = i0 + 4 * tx;
    const int P = G.pitch;
    const long long so = (long long)s * G.fsz, mo = moff(G, s);
    float *__restrict__ vx = W.vx + so;
    float *__restrict__ vy = W.vy + so;
    const float *hc = G.hc;
    float ox[4], oy[4], rp[4], rq[4];
    {
        const int j = c0 * VT_RB + 1 + w;
        if (i <= G.nx && j <= G.ny) {
            const int o = (j - 1 + HY) * P + (i - 1 + HX);
            ldv_rw<4>(vx + o, ox), ldv_rw<4>(vy + o, oy);
            ldv<4>(M.prip + mo + o, rp), ldv<4>(M.prjp + mo + o, rq);
        }
    }
    bool ok = mbar_wait(&full[0], 0) && mbar_wait(&full[1], 0);
    for (int k = 1; ok && k <= nload - 2; k++) {
        const int c = c0 - 1 + k;  // chunk computed in this pass
        const int j = c * VT_RB + 1 + w;
        float nox[4], noy[4], nrp[4], nrq[4];  // the next chunk's row, loaded while this one computes
        {
            const int jn = j + VT_RB;
            if (k < nload - 2 && i <= G.nx && jn <= G.ny) {
                const int o = (jn - 1 + HY) * P + (i - 1 + HX);
                ldv_rw<4>(vx + o, nox), ldv_rw<4>(vy + o, noy);
                ldv<4>(M.prip + mo + o, nrp), ldv<4>(M.prjp + mo + o, nrq);
            }
        }
        if (!mbar_wait(&full[(k + 1) % VT_NS], ((k + 1) / VT_NS) & 1)) {
            ok = false;
            break;
        }
        const float *prev = ring + ((k - 1) % VT_NS) * S::STAGE;
        const float *cur = ring + (k % VT_NS) * S::STAGE;
        const float *next = ring + ((k + 1) % VT_NS) * S::STAGE;
        float sxx_x[4], sxy_x[4], sxy_y[4], syy_y[4];
        {
            float X[4 * (2 * K + 1)], Y[4 * (2 * K + 1)];  // columns i - 4K .. i + 4K + 3
            const float *rx = cur + S::XX + w * S::SW + 4 * tx;
            const float *ry = cur + S::XY + w * S::SW + 4 * tx;
#pragma unroll
            for (int q = 0; q < 2 * K + 1; q++) {
                const float4 a = *reinterpret_cast<const float4 *>(rx + 4 * q);
                const float4 b = *reinterpret_cast<const float4 *>(ry + 4 * q);
                X[4 * q] = a.x, X[4 * q + 1] = a.y, X[4 * q + 2] = a.z, X[4 * q + 3] = a.w;
                Y[4 * q] = b.x, Y[4 * q + 1] = b.y, Y[4 * q + 2] = b.z, Y[4 * q + 3] = b.w;
            }
            constexpr int C = 4 * K;
#pragma unroll
            for (int cc = 0; cc < 4; cc++) {
                sxx_x[cc] = hc[1] * (X[C + cc + 1] - X[C + cc]);
                sxy_x[cc] = hc[1] * (Y[C + cc] - Y[C + cc - 1]);
#pragma unroll
                for (int m = 2; m <= ND; m++) {
                    sxx_x[cc] += hc[m] * (X[C + cc + m] - X[C + cc - m + 1]);
                    sxy_x[cc] += hc[m] * (Y[C + cc + m - 1] - Y[C + cc - m]);
                }
            }
        }
        {
            // sxy rows j - ND .. j + ND - 1, syy rows j - ND + 1 .. j + ND
            auto XY = [&](int d) {
                return *reinterpret_cast<const float4 *>(vt_row(prev, cur, next, S::XY, S::SW, w + d) + S::HXs + 4 * tx);
            };
            auto YY = [&](int d) {
                return *reinterpret_cast<const float4 *>(vt_row(prev, cur, next, S::YY, VT_TW, w + d) + 4 * tx);
            };
            float4 a1 = XY(0), a0 = XY(-1), b1 = YY(1), b0 = YY(0);
            sxy_y[0] = hc[1] * (a1.x - a0.x), sxy_y[1] = hc[1] * (a1.y - a0.y);
            sxy_y[2] = hc[1] * (a1.z - a0.z), sxy_y[3] = hc[1] * (a1.w - a0.w);
            syy_y[0] = hc[1] * (b1.x - b0.x), syy_y[1] = hc[1] * (b1.y - b0.y);
            syy_y[2] = hc[1] * (b1.z - b0.z), syy_y[3] = hc[1] * (b1.w - b0.w);
#pragma unroll
            for (int m = 2; m <= ND; m++) {
                a1 = XY(m - 1), a0 = XY(-m), b1 = YY(m), b0 = YY(-(m - 1));
                sxy_y[0] += hc[m] * (a1.x - a0.x), sxy_y[1] += hc[m] * (a1.y - a0.y);
                sxy_y[2] += hc[m] * (a1.z - a0.z), sxy_y[3] += hc[m] * (a1.w - a0.w);
                syy_y[0] += hc[m] * (b1.x - b0.x), syy_y[1] += hc[m] * (b1.y - b0.y);
                syy_y[2] += hc[m] * (b1.z - b0.z), syy_y[3] += hc[m] * (b1.w - b0.w);
            }
        }
        // chunk k-1 is read by no later pass: hand its stage back to the producer
        __syncwarp();
        if (lane == 0)
            mbar_arrive(&empty[(k - 1) % VT_NS]);
        if (i <= G.nx && j <= G.ny) {
            const int o = (j - 1 + HY) * P + (i - 1 + HX);
            v_finish<4, true>(G, W, M, s, i, j, o, mo, vx, vy, ox, oy, rp, rq, sxx_x, sxy_x, sxy_y, syy_y);
        }
#pragma unroll
        for (int cc = 0; cc < 4; cc++)
            ox[cc] = nox[cc], oy[cc] = noy[cc], rp[cc] = nrp[cc], rq[cc] = nrq[cc];
    }
    if (!ok && lane == 0 && G.fault)
        atomicOr(G.fault, 1);
}

}  // namespace sofi
