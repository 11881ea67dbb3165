// sofi_fused.cuh -- the velocity and the stress update of one time step in
// one kernel (ISO / VTI media, elastic or viscoelastic; second-order time
// stepping; no periodic edge).
//
// The plain step reads the stresses in the velocity kernel and the new
// velocities again in the stress kernel. Here each block owns a tile of
// 128 x 16 cells (32 x 8 threads, four cells per thread, two rows each):
//   1. v(n) on the tile and an ND-cell halo, from the current buffers
//      (v(n-1), s(n-1), the velocity CPML memory), into shared memory; the
//      tile's own cells also go to the next buffers with their CPML memory;
//   2. s(n) of the own cells from the shared v(n), s(n-1) of the current
//      buffers, the memory variables and the stress CPML memory (both in
//      place), into the next buffers.
// Halo cells belong to neighbouring tiles, which compute them again in the
// same launch, so the state they start from must not change during it: v,
// s and the velocity CPML memory are held twice and swapped every step (the
// host swaps the buffer sets; the post kernel and everything after it see
// the new one). Per cell the arithmetic is that of k_update_vw<ND,4> and
// k_update_sw<ND,KIND,VISCO,L,4> (the same device functions).
//
// Index ranges (ND <= 6, HG = ceil(ND/4) vectors of halo per side): region
// rows j0 - ND .. j0 + 15 + ND, columns i0 - 4 HG .. i0 + 127 + 4 HG. Rows
// outside 1 .. NY and vectors wholly outside 1 .. NX keep the ghost values of
// the current buffers (never updated); rows past NY + ND and columns past
// NX + ND feed no own cell and are not read at all. A vector that straddles
// NX is computed whole, its cells past NX replaced by their ghost values.
#pragma once
#include "sofi_dispatch.cuh"
#include "sofi_kernels.cuh"

namespace sofi {

constexpr int FU_TY = 2 * BY;  // own rows of a tile

template <int ND, int KIND, bool VISCO, int LT>
__global__ void __launch_bounds__(BX *BY, 2) k_fused(Geo G, Wave Wc, Wave Wn, Model M)
{
    constexpr int HG = (ND + 3) / 4, GPR = BX + 2 * HG;  // vectors per region row
    constexpr int RX = 4 * GPR, RY = FU_TY + 2 * ND;
    __shared__ __align__(16) float sv[2][RY][RX];
    int bx, s;
    block_xs(G, bx, s);
    const int i0 = bx * 4 * BX + 1, j0 = blockIdx.y * FU_TY + 1;
    const int tid = threadIdx.y * BX + threadIdx.x;
    if (G.step_ctr && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && tid == 0)
        *G.step_ctr += 1;
    const int P = G.pitch;
    const long long so = (long long)s * G.fsz, mo = moff(G, s);
    const float *__restrict__ sxx = Wc.sxx + so;
    const float *__restrict__ sxy = Wc.sxy + so;
    const float *__restrict__ syy = Wc.syy + so;
    // 1. velocities of the region
    for (int g = tid; g < GPR * RY; g += BX * BY) {
        const int gx = g % GPR, gy = g / GPR;
        const int i = i0 - 4 * HG + 4 * gx, j = j0 - ND + gy;
        float4 *dx_ = reinterpret_cast<float4 *>(&sv[0][gy][4 * gx]);
        float4 *dy_ = reinterpret_cast<float4 *>(&sv[1][gy][4 * gx]);
        if (j > G.ny + ND || i > G.nx + ND) {  // read by no own cell
            *dx_ = make_float4(0.f, 0.f, 0.f, 0.f), *dy_ = *dx_;
            continue;
        }
        const int o = (j - 1 + HY) * P + (i - 1 + HX);
        float ox[4], oy[4];
        ldv<4>(Wc.vx + so + o, ox), ldv<4>(Wc.vy + so + o, oy);
        if (j < 1 || j > G.ny || i > G.nx || i + 3 < 1) {  // ghost cells: their value as it stands
            *dx_ = make_float4(ox[0], ox[1], ox[2], ox[3]), *dy_ = make_float4(oy[0], oy[1], oy[2], oy[3]);
            continue;
        }
        float sxx_x[4], sxy_x[4], sxy_y[4], syy_y[4], rp[4], rq[4], nvx[4], nvy[4];
        v_derivs<ND, 4, true>(
            G, [&](int f, int dy, int dx, float *out) { ldv<4>((f == 0 ? sxx : f == 1 ? sxy : syy) + o + dy * P + dx, out); },
            sxx_x, sxy_x, sxy_y, syy_y);
        ldv<4>(M.prip + mo + o, rp), ldv<4>(M.prjp + mo + o, rq);
        const bool own = gy >= ND && gy < ND + FU_TY && gx >= HG && gx < HG + BX;
        v_compute<4, true>(G, Wc, Wn, M, s, i, j, o, mo, ox, oy, rp, rq, sxx_x, sxy_x, sxy_y, syy_y, nvx, nvy, own);
#pragma unroll
        for (int c = 0; c < 4; c++)
            if (i + c > G.nx)
                nvx[c] = ox[c], nvy[c] = oy[c];
        *dx_ = make_float4(nvx[0], nvx[1], nvx[2], nvx[3]), *dy_ = make_float4(nvy[0], nvy[1], nvy[2], nvy[3]);
        if (own) {
            float *vx = Wn.vx + so, *vy = Wn.vy + so;
            if (i + 3 <= G.nx) {
                stv<4>(vx + o, nvx), stv<4>(vy + o, nvy);
            } else {
#pragma unroll
                for (int c = 0; c < 4; c++)
                    if (i + c <= G.nx)
                        vx[o + c] = nvx[c], vy[o + c] = nvy[c];
            }
        }
    }
    __syncthreads();
    // 2. stresses of the own cells
#pragma unroll 1
    for (int r = 0; r < 2; r++) {
        const int ty = threadIdx.y + BY * r, tx = threadIdx.x;
        const int i = i0 + 4 * tx, j = j0 + ty;
        if (i > G.nx || j > G.ny)
            continue;
        const int o = (j - 1 + HY) * P + (i - 1 + HX);
        const int sy = ND + ty, sx = 4 * HG + 4 * tx;
        float vxx[4], vyx[4], vxy[4], vyy[4];
        s_derivs<ND, 4>(
            G,
            [&](int f, int dy, int dx, float *out) {
                const float4 a = *reinterpret_cast<const float4 *>(&sv[f][sy + dy][sx + dx]);
                out[0] = a.x, out[1] = a.y, out[2] = a.z, out[3] = a.w;
            },
            vxx, vyx, vxy, vyy);
        s_update<ND, KIND, VISCO, LT, 4>(G, Wc, Wn, M, s, i, j, o, mo, vxx, vyx, vxy, vyy);
    }
}

}  // namespace sofi

namespace sofi {

template <int KIND, bool VISCO>
void launch_fused_kv(const Geo &G, const Wave &Wc, const Wave &Wn, const Model &M, int nd, cudaStream_t st)
{
    const unsigned S = (unsigned)G.nshots;
    const unsigned tx = (G.nx + 4 * BX - 1) / (4 * BX), ty = (G.ny + FU_TY - 1) / FU_TY;
    const dim3 grd = G.shot_fast ? dim3(tx * S, ty, 1) : dim3(tx, ty, S), blk(BX, BY);
    const int L = VISCO ? G.L : 0;
    if (!VISCO) {
        DISPATCH_ND(nd, (k_fused<ND, KIND, false, 0><<<grd, blk, 0, st>>>(G, Wc, Wn, M)));
    } else if (L == 1) {
        DISPATCH_ND(nd, (k_fused<ND, KIND, true, 1><<<grd, blk, 0, st>>>(G, Wc, Wn, M)));
    } else if (L == 2) {
        DISPATCH_ND(nd, (k_fused<ND, KIND, true, 2><<<grd, blk, 0, st>>>(G, Wc, Wn, M)));
    } else if (L == 3) {
        DISPATCH_ND(nd, (k_fused<ND, KIND, true, 3><<<grd, blk, 0, st>>>(G, Wc, Wn, M)));
    } else {
        DISPATCH_ND(nd, (k_fused<ND, KIND, true, 0><<<grd, blk, 0, st>>>(G, Wc, Wn, M)));
    }
}

}  // namespace sofi
