// sofi_kernels.cuh -- the per-step kernels (see the overview in sofi_common.cuh).
#pragma once
#include "sofi_common.cuh"

namespace sofi {

// -------------------------------------------------------------- sources

// update_v_interior.c:49-71. Runs before the velocity kernel advances the
// step counter, so the step being computed is counter + 1. The sources and
// the model do not change during a run: the shot's source range, its first
// source's type and cell, the buoyancy there and its signal around the step
// (SigWindow) load before the wait for the previous kernel, the step number
// and the velocities after it. (static: the header is included by several
// translation units; only sofigpu.cu launches it)
__device__ __forceinline__ void force_shot(const Geo &G, const Wave &W, const Model &M, const Acq &A, int s, bool live)
{
    const float *prip = M.prip + moff(G, s), *prjp = M.prjp + moff(G, s);
    int ka = 0, kb = 0, t0 = 0;
    long long o0 = 0;
    float rx0 = 0.f, ry0 = 0.f;
    SigWindow sw{};
    if (live) {
        ka = A.src_off[s], kb = A.src_off[s + 1];
        if (ka < kb) {
            t0 = A.src_type[ka];
            o0 = cell(G, A.src_iy[ka], A.src_ix[ka]);
            rx0 = prip[o0], ry0 = prjp[o0];
            if (t0 >= 2 && t0 <= 4)
                sw.load(G.step_ctr, A.signals + (long long)ka * A.nt - 1, A.nt);
        }
    }
    pdl_begin();
    if (!live)
        return;
    const int nt = *G.step_ctr + 1;
    float *vx = W.vx + (long long)s * G.fsz, *vy = W.vy + (long long)s * G.fsz;
    for (int k = ka; k < kb; k++) {
        const int t = k == ka ? t0 : A.src_type[k];
        if (t < 2 || t > 4)
            continue;
        const long long o = k == ka ? o0 : cell(G, A.src_iy[k], A.src_ix[k]);
        const float rx = k == ka ? rx0 : prip[o], ry = k == ka ? ry0 : prjp[o];
        const float *sig = A.signals + (long long)k * A.nt - 1;  // 1-based
        float amp = (G.dt * (k == ka ? sw.at(sig, nt) : sig[nt])) / (G.dh * G.dh);
        if (t == 2)
            vx[o] += rx * amp;
        else if (t == 3)
            vy[o] += ry * amp;
        else {
            vx[o] += A.src_sin[k] * (rx * amp);
            vy[o] += A.src_cos[k] * (ry * amp);
        }
    }
}

static __global__ void k_force_src(Geo G, Wave W, Model M, Acq A)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    force_shot(G, W, M, A, s, s < G.nshots);
}

// ------------------------------------------------------- velocity update

// Velocity update, R consecutive rows per thread (the y-stencil windows of the
// R cells overlap, so σxy and σyy are loaded R + 2ND - 1 times instead of
// 2ND * R); 32-bit offsets inside a shot's fields, read-only data through the
// non-coherent cache. Force sources are added by k_force_src beforehand.
template <int ND, int R>
__global__ void __launch_bounds__(BX *BY, R == 1 ? 8 : 1) k_update_v(Geo G, Wave W, Model M)
{
    pdl_begin();
    int bx, s;
    block_xs(G, bx, s);
    const int i = bx * BX + threadIdx.x + 1;
    const int jb = (blockIdx.y * BY + threadIdx.y) * R + 1;
    // one thread advances the step counter: every kernel queued before this
    // one has read it, every kernel after it sees the step being computed
    if (G.step_ctr && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0 && threadIdx.y == 0)
        *G.step_ctr += 1;
    if (i > G.nx || jb > G.ny)
        return;
    const int P = G.pitch;
    const int ob = (jb - 1 + HY) * P + (i - 1 + HX);
    const long long so = (long long)s * G.fsz, mo = moff(G, s);
    const float *__restrict__ sxx = W.sxx + so;
    const float *__restrict__ syy = W.syy + so;
    const float *__restrict__ sxy = W.sxy + so;
    float *__restrict__ vx = W.vx + so;
    float *__restrict__ vy = W.vy + so;
    const float *hc = G.hc;
    // windows: wxy[k] = sxy(jb - ND + k), wyy[k] = syy(jb - ND + 1 + k); rows past
    // NY + ND are read by no cell of the grid and are not loaded (one row per
    // thread: the stencil reads the rows directly)
    constexpr int NW = R + 2 * ND - 1;
    float wxy[NW], wyy[NW];
    if (R > 1) {
#pragma unroll
        for (int k = 0; k < NW; k++) {
            wxy[k] = (jb - ND + k <= G.ny + ND) ? __ldg(sxy + ob + (k - ND) * P) : 0.f;
            wyy[k] = (jb - ND + 1 + k <= G.ny + ND) ? __ldg(syy + ob + (k - ND + 1) * P) : 0.f;
        }
    }
    const int xr = xside(G, i);
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int j = jb + r;
        if (j > G.ny)
            break;
        const int o = ob + r * P;
        const float ovx = vx[o], ovy = vy[o];
        const float rip = __ldg(M.prip + mo + o), rjp = __ldg(M.prjp + mo + o);
        float sxx_x, sxy_x, sxy_y, syy_y;
        if (R == 1) {
            op_v<ND>(sxx, syy, sxy, o, P, hc, sxx_x, sxy_x, sxy_y, syy_y);
        } else {
            sxx_x = hc[1] * (__ldg(sxx + o + 1) - __ldg(sxx + o));
            sxy_x = hc[1] * (__ldg(sxy + o) - __ldg(sxy + o - 1));
            sxy_y = hc[1] * (wxy[ND + r] - wxy[ND + r - 1]);
            syy_y = hc[1] * (wyy[ND + r] - wyy[ND + r - 1]);
#pragma unroll
            for (int m = 2; m <= ND; m++) {
                sxx_x += hc[m] * (__ldg(sxx + o + m) - __ldg(sxx + o - m + 1));
                sxy_x += hc[m] * (__ldg(sxy + o + m - 1) - __ldg(sxy + o - m));
                sxy_y += hc[m] * (wxy[ND + r + m - 1] - wxy[ND + r - m]);
                syy_y += hc[m] * (wyy[ND + r - 1 + m] - wyy[ND + r - m]);
            }
        }
        const int yr = yside(G, j);
        if (G.abs_type == 1) {
            if (xr) {
                int h = xr == 1 ? i : i - G.nx + G.fw2;
                long long q = ((long long)s * G.ny + (j - 1)) * G.fw2 + (h - 1);
                float ps = M.b_x_half[h - 1] * W.psi_sxx_x[q] + M.a_x_half[h - 1] * sxx_x;
                W.psi_sxx_x[q] = ps;
                sxx_x = sxx_x / M.K_x_half[h - 1] + ps;
                float py = M.b_x[h - 1] * W.psi_sxy_x[q] + M.a_x[h - 1] * sxy_x;
                W.psi_sxy_x[q] = py;
                sxy_x = sxy_x / M.K_x[h - 1] + py;
            }
            if (yr) {
                int h = yr == 1 ? j : j - G.ny + G.fw2;
                long long q = ((long long)s * G.fw2 + (h - 1)) * G.nx + (i - 1);
                float ps = M.b_y_half[h - 1] * W.psi_syy_y[q] + M.a_y_half[h - 1] * syy_y;
                W.psi_syy_y[q] = ps;
                syy_y = syy_y / M.K_y_half[h - 1] + ps;
                float py = M.b_y[h - 1] * W.psi_sxy_y[q] + M.a_y[h - 1] * sxy_y;
                W.psi_sxy_y[q] = py;
                sxy_y = sxy_y / M.K_y[h - 1] + py;
            }
        }
        float nvx = ovx + (sxx_x + sxy_y) * G.dtdh * rip;
        float nvy = ovy + (sxy_x + syy_y) * G.dtdh * rjp;
        if (G.abs_type == 2 && (xr | yr)) {
            float a = __ldg(M.absorb + mo + o);
            nvx *= a;
            nvy *= a;
        }
        vx[o] = nvx;
        vy[o] = nvy;
    }
}

// The velocity update with VW adjacent cells per thread (VW = 2 or 4; columns
// i .. i+VW-1, i = 1 mod VW): every field is read with 8- or 16-byte loads, the
// x stencils from 2K+1 vectors of the row (K = ceil(ND/VW)) and the y stencils
// one vector per row, a fraction of the load instructions of one cell per
// thread. Same arithmetic, per cell and term by term, as k_update_v.
// Reads reach columns up to i + VW(K+1) - 1 + HX - 1 of the padded row
// (< pitch for VW = 2; for VW = 4 possibly the next row's first columns); the
// values past column NX + ND only feed cells past NX, which are never stored.
// Rows j - ND .. j + ND stay inside the HY ghost rows.
template <int VW>
__device__ __forceinline__ void ldv(const float *p, float *out)
{
    if (VW == 1) {
        out[0] = __ldg(p);
    } else if (VW == 4) {
        const float4 a = __ldg(reinterpret_cast<const float4 *>(p));
        out[0] = a.x, out[1] = a.y, out[2] = a.z, out[3] = a.w;
    } else {
        const float2 a = __ldg(reinterpret_cast<const float2 *>(p));
        out[0] = a.x, out[1] = a.y;
    }
}

template <int VW>
__device__ __forceinline__ void ldv_rw(const float *p, float *out)  // arrays this kernel writes
{
    if (VW == 1) {
        out[0] = *p;
    } else if (VW == 4) {
        const float4 a = *reinterpret_cast<const float4 *>(p);
        out[0] = a.x, out[1] = a.y, out[2] = a.z, out[3] = a.w;
    } else {
        const float2 a = *reinterpret_cast<const float2 *>(p);
        out[0] = a.x, out[1] = a.y;
    }
}

// VW-wide loads of operands each thread reads once, kept out of L1 (16-byte
// loads; narrower ones are plain) so that the stencil rows the threads of a
// block share stay there: read-only data through the non-coherent path, and
// data the kernel writes (each cell by the thread that read it).
template <int VW>
__device__ __forceinline__ void ldv_once(const float *p, float *out)
{
    if (VW == 4)
        asm("ld.global.nc.L1::no_allocate.v4.f32 {%0, %1, %2, %3}, [%4];"
            : "=f"(out[0]), "=f"(out[1]), "=f"(out[2]), "=f"(out[3])
            : "l"(p));
    else
        ldv<VW>(p, out);
}

template <int VW>
__device__ __forceinline__ void ldv_rw_once(const float *p, float *out)
{
    if (VW == 4)
        asm("ld.global.L1::no_allocate.v4.f32 {%0, %1, %2, %3}, [%4];"
            : "=f"(out[0]), "=f"(out[1]), "=f"(out[2]), "=f"(out[3])
            : "l"(p));
    else
        ldv_rw<VW>(p, out);
}

template <int VW>
__device__ __forceinline__ void stv(float *p, const float *v)
{
    if (VW == 1)
        *p = v[0];
    else if (VW == 4)
        *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
    else
        *reinterpret_cast<float2 *>(p) = make_float2(v[0], v[1]);
}

// The end of a velocity update of VW adjacent cells (columns i .. i+VW-1, row
// j, padded offset o) from the four stress derivatives: CPML stretch and
// memory (cpml_update.c), vx/vy update (wavefield_update_v.c / _ac.c),
// damping frame (update_v_abs.c) and the store of the cells i + c <= NX.
// ox/oy: the old velocities, rp/rq: the cells' rip / rjp.
template <int VW, bool SXY, bool FWI = false>
__device__ __forceinline__ void v_compute(const Geo &G, const Wave &Wr, const Wave &Ww, const Model &M, int s, int i,
                                          int j, int o, long long mo, const float *ox, const float *oy,
                                          const float *rp, const float *rq, const float *sxx_x, const float *sxy_x,
                                          const float *sxy_y, const float *syy_y, float *nvx, float *nvy, bool own)
{
    const int yr = yside(G, j);
    const bool xframe = i <= G.gx2 || i + VW - 1 > G.gx3;  // any of the cells in a left/right frame
#pragma unroll
    for (int c = 0; c < VW; c++) {
        const int ic = i + c;
        float fx = sxx_x[c], fxy = sxy_x[c], fyx = sxy_y[c], fy = syy_y[c];
        const int xr = xframe ? xside(G, ic) : 0;
        if (G.abs_type == 1 && ic <= G.nx) {
            if (xr) {
                int h = xr == 1 ? ic : ic - G.nx + G.fw2;
                long long q = ((long long)s * G.ny + (j - 1)) * G.fw2 + (h - 1);
                float ps = M.b_x_half[h - 1] * Wr.psi_sxx_x[q] + M.a_x_half[h - 1] * fx;
                if (own)
                    Ww.psi_sxx_x[q] = ps;
                fx = fx / M.K_x_half[h - 1] + ps;
                if (SXY) {
                    float py = M.b_x[h - 1] * Wr.psi_sxy_x[q] + M.a_x[h - 1] * fxy;
                    if (own)
                        Ww.psi_sxy_x[q] = py;
                    fxy = fxy / M.K_x[h - 1] + py;
                }
            }
            if (yr) {
                int h = yr == 1 ? j : j - G.ny + G.fw2;
                long long q = ((long long)s * G.fw2 + (h - 1)) * G.nx + (ic - 1);
                float ps = M.b_y_half[h - 1] * Wr.psi_syy_y[q] + M.a_y_half[h - 1] * fy;
                if (own)
                    Ww.psi_syy_y[q] = ps;
                fy = fy / M.K_y_half[h - 1] + ps;
                if (SXY) {
                    float py = M.b_y[h - 1] * Wr.psi_sxy_y[q] + M.a_y[h - 1] * fyx;
                    if (own)
                        Ww.psi_sxy_y[q] = py;
                    fyx = fyx / M.K_y[h - 1] + py;
                }
            }
        }
        if (SXY) {
            if (FWI && own && ic <= G.nx) {
                Ww.fa_x[(long long)s * G.fsz + o + c] = rp[c] * (fx + fyx) / G.dh;
                Ww.fa_y[(long long)s * G.fsz + o + c] = rq[c] * (fxy + fy) / G.dh;
            }
            nvx[c] = ox[c] + (fx + fyx) * G.dtdh * rp[c];
            nvy[c] = oy[c] + (fxy + fy) * G.dtdh * rq[c];
        } else {
            nvx[c] = ox[c] + fx * G.dtdh * rp[c];
            nvy[c] = oy[c] + fy * G.dtdh * rq[c];
        }
        if (G.abs_type == 2 && (xr | yr)) {
            float a = __ldg(M.absorb + mo + o + c);
            nvx[c] *= a;
            nvy[c] *= a;
        }
    }
}

template <int VW, bool SXY, bool FWI = false>
__device__ __forceinline__ void v_finish(const Geo &G, const Wave &W, const Model &M, int s, int i, int j, int o,
                                         long long mo, float *__restrict__ vx, float *__restrict__ vy,
                                         const float *ox, const float *oy, const float *rp, const float *rq,
                                         const float *sxx_x, const float *sxy_x, const float *sxy_y,
                                         const float *syy_y)
{
    float nvx[VW], nvy[VW];
    v_compute<VW, SXY, FWI>(G, W, W, M, s, i, j, o, mo, ox, oy, rp, rq, sxx_x, sxy_x, sxy_y, syy_y, nvx, nvy, true);
    if (i + VW - 1 <= G.nx) {
        stv<VW>(vx + o, nvx);
        stv<VW>(vy + o, nvy);
    } else {
#pragma unroll
        for (int c = 0; c < VW; c++)
            if (i + c <= G.nx)
                vx[o + c] = nvx[c], vy[o + c] = nvy[c];
    }
}

// A backward step of an FWI pass, before the velocity update of VW adjacent
// cells (columns i .., row j; ox / oy their velocities): the adjoint signals
// of the receivers at a cell in the reference's order (update_v_interior.c:
// 72-90, adjoint type 1-3), then pvxp1 / pvyp1 (wavefield_update_v.c:36-41:
// the injected velocity, or with VELOCITY = 0 its running sum times DT) and
// the density term of calc_conv.c:49-51 against forward slot NT - nt + 1.
// Each product and sum is rounded on its own, as the reference evaluates
// them. The step number comes from FwiDev::bstep, which the previous step's
// correlation kernel wrote: this kernel advances the step counter itself.
template <int VW>
__device__ __forceinline__ void bwd_cells(const Geo &G, const FwiDev &F, int i, int j, float *ox, float *oy)
{
    const int nt = *F.bstep + 1;
    const long long n = (long long)G.nx * G.ny;
    const float *slot = F.store + (long long)(F.nt - nt - *F.base) * 5 * n;
#pragma unroll
    for (int c = 0; c < VW; c++) {
        if (i + c > G.nx)
            continue;
        const long long q = (long long)(j - 1) * G.nx + (i + c - 1);
        const int k = F.cell_map[q] - 1;
        if (k >= 0)
            for (int r = F.cell_off[k]; r < F.cell_off[k + 1]; r++) {
                const int l = F.cell_rec[r];
                if (F.adjoint == 1 || F.adjoint == 3)
                    ox[c] += F.adj[(long long)l * F.nt + (nt - 1)];
                if (F.adjoint == 1 || F.adjoint == 2)
                    oy[c] += F.adj[((long long)F.ntr + l) * F.nt + (nt - 1)];
            }
        float px = ox[c], py = oy[c];
        if (!F.velocity) {
            px = __fadd_rn(F.px[q], __fmul_rn(px, G.dt));
            py = __fadd_rn(F.py[q], __fmul_rn(py, G.dt));
            F.px[q] = px, F.py[q] = py;
        }
        const float t = __fadd_rn(__fmul_rn(px, slot[q]), __fmul_rn(py, slot[n + q]));
        F.g_rhos[q] = __fadd_rn(F.g_rhos[q], __fmul_rn(-G.dt, t));
    }
}

// The stress derivatives of VW adjacent cells for the velocity update
// (op_v_fdN, initfd.c:97-183, unscaled): ld(f, dy, dx, out) loads VW values
// of sxx (f = 0), sxy (1) or syy (2) at row j + dy, columns i + dx ..
// i + dx + VW - 1. The 4th-order kernels use it; vw_tile writes the same
// expressions out inline (through a loader they cost the 64-register
// four-cell kernel a spill).
template <int ND, int VW, bool SXY, class LD>
__device__ __forceinline__ void v_derivs(const Geo &G, LD ld, float *sxx_x, float *sxy_x, float *sxy_y, float *syy_y)
{
    constexpr int K = (ND + VW - 1) / VW;
    constexpr int NXS = VW * (2 * K + 1);  // stencil row: columns i - VW K .. i + VW K + VW - 1
    const float *hc = G.hc;
    {
        float X[NXS], Y[NXS];  // X[k] = sxx(j, i - VW K + k), Y[k] = sxy(j, i - VW K + k)
#pragma unroll
        for (int q = 0; q < 2 * K + 1; q++) {
            ld(0, 0, VW * (q - K), X + VW * q);
            if (SXY)
                ld(1, 0, VW * (q - K), Y + VW * q);
        }
        constexpr int C = VW * K;  // index of column i
#pragma unroll
        for (int c = 0; c < VW; c++) {
            sxx_x[c] = hc[1] * (X[C + c + 1] - X[C + c]);
            sxy_x[c] = SXY ? hc[1] * (Y[C + c] - Y[C + c - 1]) : 0.f;
#pragma unroll
            for (int m = 2; m <= ND; m++) {
                sxx_x[c] += hc[m] * (X[C + c + m] - X[C + c - m + 1]);
                if (SXY)
                    sxy_x[c] += hc[m] * (Y[C + c + m - 1] - Y[C + c - m]);
            }
        }
    }
    {
        // y stencils: sxy rows j - ND .. j + ND - 1, syy rows j - ND + 1 .. j + ND
        float a1[VW], a0[VW], b1[VW], b0[VW];
        if (SXY)
            ld(1, 0, 0, a1), ld(1, -1, 0, a0);
        ld(2, 1, 0, b1), ld(2, 0, 0, b0);
#pragma unroll
        for (int c = 0; c < VW; c++) {
            sxy_y[c] = SXY ? hc[1] * (a1[c] - a0[c]) : 0.f;
            syy_y[c] = hc[1] * (b1[c] - b0[c]);
        }
#pragma unroll
        for (int m = 2; m <= ND; m++) {
            if (SXY)
                ld(1, m - 1, 0, a1), ld(1, -m, 0, a0);
            ld(2, m, 0, b1), ld(2, -(m - 1), 0, b0);
#pragma unroll
            for (int c = 0; c < VW; c++) {
                if (SXY)
                    sxy_y[c] += hc[m] * (a1[c] - a0[c]);
                syy_y[c] += hc[m] * (b1[c] - b0[c]);
            }
        }
    }
}

// SXY = false: the acoustic update (wavefield_update_v_ac.c), which has no
// sxy: vx += sxx_x * DT/DH * rip, vy += syy_y * DT/DH * rjp (sxx and syy are
// one pressure array); VW may then also be 1.
// TBX: threads of a block in x (BX, or 8 for narrow grids: 32 columns by 32
// rows per block of four-cell threads, so a 400-cell row leaves 4 % of the
// last block idle instead of 22 %).
template <int ND, int VW, bool SXY, bool FWI = false, int TBX = BX, bool BWD = false>
__device__ __forceinline__ void vw_tile(const Geo &G, const Wave &W, const Model &M, const uint3 b,
                                        const FwiDev *F = nullptr)
{
    constexpr int K = (ND + VW - 1) / VW;
    constexpr int NXS = VW * (2 * K + 1);  // stencil row: columns i - VW K .. i + VW K + VW - 1
    constexpr int TBY = BX * BY / TBX;
    int bx, s;
    block_xs(G, b, bx, s);
    const int i = (bx * TBX + threadIdx.x) * VW + 1;
    const int j = b.y * TBY + threadIdx.y + 1;
    if (G.step_ctr && b.x == 0 && b.y == 0 && b.z == 0 && threadIdx.x == 0 && threadIdx.y == 0)
        *G.step_ctr += 1;
    if (i > G.nx || j > G.ny)
        return;
    const int P = G.pitch;
    const int o = (j - 1 + HY) * P + (i - 1 + HX);  // VW-aligned: HX = 8, P % 32 == 0, i - 1 = 0 mod VW
    const long long so = (long long)s * G.fsz, mo = moff(G, s);
    const float *__restrict__ sxx = W.sxx + so;
    const float *__restrict__ syy = W.syy + so;
    const float *__restrict__ sxy = W.sxy + so;
    const float *hc = G.hc;
    float sxx_x[VW], sxy_x[VW], sxy_y[VW], syy_y[VW];
    {
        float X[NXS], Y[NXS];  // X[k] = sxx(j, i - VW K + k), Y[k] = sxy(j, i - VW K + k)
#pragma unroll
        for (int q = 0; q < 2 * K + 1; q++) {
            ldv<VW>(sxx + o + VW * (q - K), X + VW * q);
            if (SXY)
                ldv<VW>(sxy + o + VW * (q - K), Y + VW * q);
        }
        constexpr int C = VW * K;  // index of column i
#pragma unroll
        for (int c = 0; c < VW; c++) {
            sxx_x[c] = hc[1] * (X[C + c + 1] - X[C + c]);
            sxy_x[c] = SXY ? hc[1] * (Y[C + c] - Y[C + c - 1]) : 0.f;
#pragma unroll
            for (int m = 2; m <= ND; m++) {
                sxx_x[c] += hc[m] * (X[C + c + m] - X[C + c - m + 1]);
                if (SXY)
                    sxy_x[c] += hc[m] * (Y[C + c + m - 1] - Y[C + c - m]);
            }
        }
    }
    {
        // y stencils: sxy rows j - ND .. j + ND - 1, syy rows j - ND + 1 .. j + ND
        float a1[VW], a0[VW], b1[VW], b0[VW];
        if (SXY)
            ldv<VW>(sxy + o, a1), ldv<VW>(sxy + o - P, a0);
        ldv<VW>(syy + o + P, b1), ldv<VW>(syy + o, b0);
#pragma unroll
        for (int c = 0; c < VW; c++) {
            sxy_y[c] = SXY ? hc[1] * (a1[c] - a0[c]) : 0.f;
            syy_y[c] = hc[1] * (b1[c] - b0[c]);
        }
#pragma unroll
        for (int m = 2; m <= ND; m++) {
            if (SXY)
                ldv<VW>(sxy + o + (m - 1) * P, a1), ldv<VW>(sxy + o - m * P, a0);
            ldv<VW>(syy + o + m * P, b1), ldv<VW>(syy + o - (m - 1) * P, b0);
#pragma unroll
            for (int c = 0; c < VW; c++) {
                if (SXY)
                    sxy_y[c] += hc[m] * (a1[c] - a0[c]);
                syy_y[c] += hc[m] * (b1[c] - b0[c]);
            }
        }
    }
    float *__restrict__ vx = W.vx + so;
    float *__restrict__ vy = W.vy + so;
    float ox[VW], oy[VW], rp[VW], rq[VW];
    ldv_rw_once<VW>(vx + o, ox), ldv_rw_once<VW>(vy + o, oy);
    ldv_once<VW>(M.prip + mo + o, rp), ldv_once<VW>(M.prjp + mo + o, rq);
    if constexpr (BWD)
        bwd_cells<VW>(G, *F, i, j, ox, oy);
    v_finish<VW, SXY, FWI>(G, W, M, s, i, j, o, mo, vx, vy, ox, oy, rp, rq, sxx_x, sxy_x, sxy_y, syy_y);
}

// FWI: the forward run of an FWI gradient pass also writes the gradient
// quantities (Wave::fa_x / fa_y); a separate instantiation, so that the plain
// kernels carry no trace of it
template <int ND, int VW, bool SXY = true, bool FWI = false, int TBX = BX>
__global__ void __launch_bounds__(BX *BY, VW == 4 ? 4 : 1) k_update_vw(Geo G, Wave W, Model M)
{
    pdl_begin();
    vw_tile<ND, VW, SXY, FWI, TBX>(G, W, M, blockIdx);
}

// A backward step of an FWI pass: the adjoint injection and the density term
// (bwd_cells) in the velocity kernel, VW = 4, 2 or 1 cells per thread; the
// four-cell form at three blocks per SM (at four it spills 36 bytes)
template <int ND, int VW>
__global__ void __launch_bounds__(BX *BY, VW == 4 ? 3 : 1) k_update_vw_bwd(Geo G, Wave W, Model M, FwiDev F)
{
    pdl_begin();
    vw_tile<ND, VW, true, false, BX, true>(G, W, M, blockIdx, &F);
}

// Periodic x (BOUNDARY = 1): ghost columns copy the opposite edge, as the one-
// rank exchange_v / exchange_s do (every column the stencils read is covered).
static __global__ void k_wrap_x(Geo G, float *a, float *b, float *c, int nd)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
    int s = blockIdx.y;
    if (j > G.ny)
        return;
    float *f[3] = {a, b, c};
    for (int t = 0; t < 3; t++) {
        if (!f[t])
            continue;
        float *x = f[t] + (long long)s * G.fsz;
        for (int l = 1; l <= nd + 1; l++) {
            x[cell(G, j, G.nx + l)] = x[cell(G, j, l)];
            x[cell(G, j, 1 - l)] = x[cell(G, j, G.nx - l + 1)];
        }
    }
}

// --------------------------------------------------------- stress update

// The acquisition of a flagged cell's post work (below), loaded by
// k_update_s_post before it waits for the velocity kernel: no kernel writes the
// acquisition arrays. Bit b of smask: source ka + b of the shot is at the cell
// (a shot has at most 8 sources here); kr: the cell's first receiver (-1:
// none), then positions rr .. r1 - 1 of the column's receiver list are left
// to search for more. Set for the cells whose flag has a bit, and read only
// under that bit.
struct CellAcq {
    unsigned smask;
    int ka, kr, rr, r1;
    SigWindow sw;  // the cell's first source's signal around this step
};

__device__ __forceinline__ CellAcq cell_acq(const Geo &G, const Acq &A, int s, int i, int j, unsigned flag)
{
    CellAcq c{0u, 0, -1, 0, 0};
    if (flag & 1) {
        c.ka = A.src_off[s];
        const int kb = A.src_off[s + 1];
        for (int k = c.ka; k < kb; k++)
            if (A.src_ix[k] == i && A.src_iy[k] == j)
                c.smask |= 1u << (k - c.ka);
        if (c.smask)
            c.sw.load(G.step_ctr, A.signals + (long long)(c.ka + __ffs(c.smask) - 1) * A.nt - 1, A.nt);
    }
    if (flag & 2) {
        const int *roff = A.rec_col_off + (long long)s * (G.nx + 1);
        int r = roff[i - 1];
        c.r1 = roff[i];
        for (; r < c.r1; r++) {
            const int k = A.rec_col_idx[r];
            if (A.rec_iy[k] == j) {
                c.kr = k;
                break;
            }
        }
        c.rr = r + 1;
    }
    return c;
}

// seismo_ssg.c:28-67 for receiver k at the cell (p after the sources).
__device__ __forceinline__ void sample_cell(const Geo &G, const Model &M, const Acq &A, int k, int o, long long mo,
                                            int ins, float nxx, float nyy, float vxo, float vyo, float vxx,
                                            float vyx, float vxy, float vyy)
{
    const int seismo = G.seismo;
    float *sec = A.sec + (long long)k * 5 * A.ns + (ins - 1);
    if (seismo == 3 || seismo == 4) {
        sec[3 * A.ns] = (vxx + vyy) * sqrtf(M.ppi[mo + o]);
        sec[4 * A.ns] = (vxy - vyx) * sqrtf(M.pu[mo + o]);
    }
    if (seismo == 1 || seismo == 4) {
        sec[0] = vxo;
        sec[A.ns] = vyo;
    }
    if (seismo == 2 || seismo == 4) {
        float p = -nxx - nyy;
        if (seismo == 2) {
            sec[2 * A.ns] = p;
        } else {
            float ppi = M.ppi[mo + o], pu = M.pu[mo + o];
            sec[2 * A.ns] = ((3.0f * ppi - 4.0f * pu) / (2.0f * ppi - 2.0f * pu)) * p / 3.0f;
        }
    }
}

// k_post's work at cell (j, i) of shot s, done by the thread that has just
// updated and stored its stresses (nxx, nyy in sxx[o], syy[o]) from the
// CPML-stretched velocity derivatives: psource.c's explosive sources of step
// nt in source order (time_loop.c:248-253), then the seismograms of
// seismo_ssg.c:28-67 at the cell's receivers (div / curl from the
// derivatives, p after the sources) and the NaN probe of time_loop.c:44-47 --
// what post_column does for the cell, term by term. (vxo, vyo): the cell's
// velocities, which the stress update has loaded; ca: its acquisition.
__device__ __forceinline__ void post_cell(const Geo &G, const Model &M, const Acq &A, int s, int i, int j, int o,
                                          long long mo, float *sxx, float *syy, float nxx, float nyy, float vxo,
                                          float vyo, float vxx, float vyx, float vxy, float vyy, unsigned flag,
                                          const CellAcq &ca)
{
    const bool probe = i == (G.nx / 2 > 0 ? G.nx / 2 : 1) && j == (G.ny / 2 > 0 ? G.ny / 2 : 1);
    if (!flag && !probe)
        return;
    const int nt = *G.step_ctr;  // the velocity kernel of this step advanced it
    // ca is only read under the flag bits (it is not set for other cells)
    for (unsigned m = (flag & 1) ? ca.smask : 0u; m; m &= m - 1) {  // the shot's last source is explosive
        const int NT = A.nt;
        const int k = ca.ka + __ffs(m) - 1;
        const float *sig = A.signals + (long long)k * NT - 1;  // 1-based
        // the first source's samples from the window loaded before the wait
        const bool first = m == ca.smask;
        auto sg = [&](int n) { return first ? ca.sw.at(sig, n) : sig[n]; };
        float amp = 0.0f;
        const float d2 = 2.0f * G.dh * G.dh;
        if (NT >= 2) {
            if (nt == 1)
                amp = sg(2) / d2;
            else if (nt < NT)
                amp = (sg(nt + 1) - sg(nt - 1)) / d2;
            else
                amp = -sg(nt - 1) / d2;
        }
        nxx += amp;
        nyy += amp;
        sxx[o] = nxx;
        syy[o] = nyy;
    }
    const int seismo = G.seismo;
    const int ins = (seismo && G.ndt > 0 && nt % G.ndt == 0 && nt < A.nt) ? nt / G.ndt : 0;
    if ((flag & 2) && ins && ca.kr >= 0) {
        sample_cell(G, M, A, ca.kr, o, mo, ins, nxx, nyy, vxo, vyo, vxx, vyx, vxy, vyy);
        for (int r = ca.rr; r < ca.r1; r++) {
            const int k = A.rec_col_idx[r];
            if (A.rec_iy[k] == j)
                sample_cell(G, M, A, k, o, mo, ins, nxx, nyy, vxo, vyo, vxx, vyx, vxy, vyy);
        }
    }
    if (probe && isnan(vyo) && A.status[s] == 0)
        A.status[s] = nt;
}

// Isotropic and VTI stress update, one thread per cell (wavefield_update_s_el.c,
// _visc.c, _el_vti.c, _visc_VTI.c). Viscoelastic modulus defects are the
// stored base (modulus * tau) times peta[l]; LT > 0 fixes the number of
// mechanisms at compile time so every memory variable is loaded up front.
// POST (k_update_s_post): the cell's share of k_post as well -- explosive
// sources, seismograms, the NaN probe -- for steps without a free surface or
// moment-tensor sources, so that the step needs no post kernel.
// POST: pflag and ca are the cell's flags and acquisition (cell_acq).
// FWI (EL_ISO, a stored step of an FWI forward run with VELOCITY = 1,
// Wave::fstore set): also the store slot, as s_update writes it.
template <int ND, int KIND, bool VISCO, int LT, bool POST, bool FWI = false>
__device__ __forceinline__ void s_one(const Geo &G, const Wave &W, const Model &M, const Acq &A, unsigned pflag,
                                      const CellAcq &ca)
{
    int bx, s;
    block_xs(G, bx, s);
    const int i = bx * BX + threadIdx.x + 1;
    const int j = blockIdx.y * BY + threadIdx.y + 1;
    if (i > G.nx || j > G.ny)
        return;
    const int P = G.pitch;
    const int o = (j - 1 + HY) * P + (i - 1 + HX);
    const long long so = (long long)s * G.fsz, mo = moff(G, s);
    float *__restrict__ sxx = W.sxx + so;
    float *__restrict__ syy = W.syy + so;
    float *__restrict__ sxy = W.sxy + so;
    const float *__restrict__ vx = W.vx + so;
    const float *__restrict__ vy = W.vy + so;
    const float oxx = sxx[o], oyy = syy[o], oxy = sxy[o];
    float m0, m1, m2, m3 = 0.f, b0 = 0.f, b1 = 0.f, b2 = 0.f, b3 = 0.f;
    if (KIND == ISO) {
        m0 = __ldg(M.g + mo + o), m1 = __ldg(M.f + mo + o), m2 = __ldg(M.fipjp + mo + o);
        if (VISCO)
            b0 = __ldg(M.db + mo + o), b1 = __ldg(M.eb + mo + o), b2 = __ldg(M.dipb + mo + o);
    } else {
        m0 = __ldg(M.c11 + mo + o), m1 = __ldg(M.c13 + mo + o), m2 = __ldg(M.c33 + mo + o);
        m3 = __ldg(M.c55ipjp + mo + o);
        if (VISCO)
            b0 = __ldg(M.c11b + mo + o), b1 = __ldg(M.c13b + mo + o), b2 = __ldg(M.c33b + mo + o),
            b3 = __ldg(M.c55ipjpb + mo + o);
    }
    constexpr int LN = LT > 0 ? LT : MAXL;
    const int L = LT > 0 ? LT : G.L;
    float *__restrict__ wr = W.r + (long long)s * G.L * G.fsz;
    float *__restrict__ wp = W.p + (long long)s * G.L * G.fsz;
    float *__restrict__ wq = W.q + (long long)s * G.L * G.fsz;
    float rr[LN], pp[LN], qq[LN];
    if (VISCO) {
#pragma unroll
        for (int l = 0; l < LN; l++) {
            if (l < L) {
                long long lo = (long long)l * G.fsz + o;
                rr[l] = wr[lo], pp[l] = wp[lo], qq[l] = wq[lo];
            }
        }
    }
    float vxx, vyx, vxy, vyy;
    {
        const float *hc = G.hc;
        vxx = hc[1] * (__ldg(vx + o) - __ldg(vx + o - 1));
        vyx = hc[1] * (__ldg(vy + o + 1) - __ldg(vy + o));
        vxy = hc[1] * (__ldg(vx + o + P) - __ldg(vx + o));
        vyy = hc[1] * (__ldg(vy + o) - __ldg(vy + o - P));
#pragma unroll
        for (int m = 2; m <= ND; m++) {
            vxx += hc[m] * (__ldg(vx + o + m - 1) - __ldg(vx + o - m));
            vyx += hc[m] * (__ldg(vy + o + m) - __ldg(vy + o - m + 1));
            vxy += hc[m] * (__ldg(vx + o + m * P) - __ldg(vx + o - (m - 1) * P));
            vyy += hc[m] * (__ldg(vy + o + (m - 1) * P) - __ldg(vy + o - m * P));
        }
        vxx *= G.dhi, vyx *= G.dhi, vxy *= G.dhi, vyy *= G.dhi;
    }
    const int xr = xside(G, i), yr = yside(G, j);
    if (G.abs_type == 1)
        cpml_s(G, W, M, s, i, j, xr, yr, vxx, vyx, vxy, vyy, true);
    float u1, u2, u3;
    if (KIND == ISO) {
        u1 = m2 * (vyx + vxy);
        float gd = m0 * (vxx + vyy);
        u2 = gd - 2.0f * m1 * vyy;
        u3 = gd - 2.0f * m1 * vxx;
        if (FWI && !VISCO && W.fstore) {
            const long long n = (long long)G.nx * G.ny;
            float *slot = W.fstore + (long long)(*G.step_ctr - 1 - *W.fbase) * 5 * n +
                          ((long long)(j - 1) * G.nx + (i - 1));
            slot[0] = W.fa_x[so + o], slot[n] = W.fa_y[so + o];
            slot[2 * n] = u2 / G.dt, slot[3 * n] = u3 / G.dt, slot[4 * n] = u1 / G.dt;
        }
    } else {
        u1 = m3 * (vxy + vyx);
        u2 = m0 * vxx + m1 * vyy;
        u3 = m1 * vxx + m2 * vyy;
    }
    if (VISCO) {
        float sro = 0.f, spo = 0.f, sqo = 0.f, sr = 0.f, sp = 0.f, sq = 0.f;
#pragma unroll
        for (int l = 0; l < LN; l++) {
            if (l < L) {
                float r = rr[l], p = pp[l], q = qq[l];
                sro += r, spo += p, sqo += q;
                float pe = M.peta[l], bb = M.bip[l], cc = M.cip[l];
                if (KIND == ISO) {
                    float dip = b2 * pe, d = b0 * pe, e = b1 * pe;
                    r = bb * (r * cc - dip * (vxy + vyx));
                    p = bb * (p * cc - e * (vxx + vyy) + 2.0f * d * vyy);
                    q = bb * (q * cc - e * (vxx + vyy) + 2.0f * d * vxx);
                } else {
                    r = bb * (r * cc - (b3 * pe) * (vxy + vyx));
                    p = bb * (p * cc - (b0 * pe) * vxx - (b1 * pe) * vyy);
                    q = bb * (q * cc - (b1 * pe) * vxx - (b2 * pe) * vyy);
                }
                long long lo = (long long)l * G.fsz + o;
                wr[lo] = r, wp[lo] = p, wq[lo] = q;
                sr += r, sp += p, sq += q;
            }
        }
        u1 += G.dthalbe * (sro + sr);
        u2 += G.dthalbe * (spo + sp);
        u3 += G.dthalbe * (sqo + sq);
    }
    float nxy = oxy + u1, nxx = oxx + u2, nyy = oyy + u3;
    if (G.abs_type == 2 && (xr | yr)) {
        float a = __ldg(M.absorb + mo + o);
        nxy *= a, nyy *= a, nxx *= a;
    }
    sxy[o] = nxy;
    sxx[o] = nxx;
    syy[o] = nyy;
    if (POST)
        post_cell(G, M, A, s, i, j, o, mo, sxx, syy, nxx, nyy, __ldg(vx + o), __ldg(vy + o), vxx, vyx, vxy, vyy,
                  pflag, ca);
}

template <int ND, int KIND, bool VISCO, int LT>
__global__ void __launch_bounds__(BX *BY) k_update_s(Geo G, Wave W, Model M)
{
    pdl_begin();
    const Acq none{};  // not read without POST
    s_one<ND, KIND, VISCO, LT, false>(G, W, M, none, 0u, CellAcq{});
}

// The cell's flags and acquisition load before the wait for the velocity
// kernel, so that a source's or a receiver's cell, the slowest threads of a
// launch-bound grid, has fewer dependent memory round trips after it. The
// acquisition waits in shared memory (a slot per thread), not in registers
// held across the stress update; at 48 registers (five blocks per SM) the
// elastic kernels do not spill, and a 400 x 400 grid is still one wave.
template <int ND, int KIND, bool VISCO, int LT>
__global__ void __launch_bounds__(BX *BY, 5) k_update_s_post(Geo G, Wave W, Model M, Acq A)
{
    __shared__ CellAcq slot[BX * BY];
    int bx, s;
    block_xs(G, bx, s);
    const int i = bx * BX + threadIdx.x + 1, j = blockIdx.y * BY + threadIdx.y + 1;
    CellAcq &ca = slot[threadIdx.y * BX + threadIdx.x];
    unsigned flag = 0;
    if (i <= G.nx && j <= G.ny) {
        flag = __ldg(A.cell_flag + ((long long)s * G.ny + (j - 1)) * G.nx + (i - 1));
        if (flag)
            ca = cell_acq(G, A, s, i, j, flag);
    }
    pdl_begin();
    s_one<ND, KIND, VISCO, LT, true>(G, W, M, A, flag, ca);
}

// A backward step of an FWI pass without a free surface, after the stress
// update of VW adjacent cells: calc_conv.c:34-71's lambda and mu terms
// against forward slot NT - nt + 1, formed in double and rounded into the
// float sums as the reference evaluates them (k_fwi_conv's arithmetic), from
// the stresses this thread has just stored. The reference divides by
// (lamss + muss)^2 and muss^2; their double reciprocals (FwiDev::rc) multiply.
template <int VW>
__device__ __forceinline__ void bwd_conv(const Geo &G, const FwiDev &F, const Model &M, const float *sxx,
                                         const float *syy, const float *sxy, int i, int j, int o, long long mo)
{
    const int nt = *G.step_ctr;
    const long long n = (long long)G.nx * G.ny;
    const float *slot = F.store + (long long)(F.nt - nt - *F.base) * 5 * n;
    const double mDT = -(double)G.dt;
#pragma unroll
    for (int c = 0; c < VW; c++) {
        if (i + c > G.nx)
            continue;
        const long long q = (long long)(j - 1) * G.nx + (i + c - 1);
        const float fx = slot[2 * n + q], fy = slot[3 * n + q], fu = slot[4 * n + q];
        const float xx = sxx[o + c], yy = syy[o + c], xy = sxy[o + c];
        const float sum_f = __fmul_rn(__fadd_rn(fx, fy), __fadd_rn(xx, yy));
        F.g_lam[q] = (float)__dadd_rn((double)F.g_lam[q], __dmul_rn(__dmul_rn(mDT, F.rc[q]), (double)sum_f));
        if (M.pu[mo + o + c] > 0.0f) {
            const double r_mm = F.rc[n + q], r_lm2 = F.rc[2 * n + q];
            const double t1 = __dmul_rn(r_mm, (double)__fmul_rn(fu, xy));
            const double t2 = __dmul_rn(__dmul_rn(0.25, (double)sum_f), r_lm2);
            const double t3 = __dmul_rn(__dmul_rn(0.25, (double)__fmul_rn(__fsub_rn(fx, fy), __fsub_rn(xx, yy))), r_mm);
            F.g_mu[q] = (float)__dadd_rn((double)F.g_mu[q], __dmul_rn(mDT, __dadd_rn(__dadd_rn(t1, t2), t3)));
        }
    }
}

// The same for the steps of an FWI pass (EL_ISO, one shot): a forward step
// also writes the store slot (s_one's FWI); a backward step without a free
// surface then adds the lambda / mu correlation from the stresses the cell
// holds after the post work (bwd_conv) and records the step it completes for
// the next backward velocity kernel.
template <int ND, bool BWD>
__global__ void __launch_bounds__(BX *BY, 4) k_update_s_post_fwi(Geo G, Wave W, Model M, Acq A, FwiDev F)
{
    __shared__ CellAcq slot[BX * BY];
    const int i = blockIdx.x * BX + threadIdx.x + 1, j = blockIdx.y * BY + threadIdx.y + 1;
    CellAcq &ca = slot[threadIdx.y * BX + threadIdx.x];
    unsigned flag = 0;
    if (i <= G.nx && j <= G.ny) {
        flag = __ldg(A.cell_flag + (long long)(j - 1) * G.nx + (i - 1));
        if (flag)
            ca = cell_acq(G, A, 0, i, j, flag);
    }
    pdl_begin();
    if (BWD && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0)
        *F.bstep = *G.step_ctr;
    s_one<ND, ISO, false, 0, true, !BWD>(G, W, M, A, flag, ca);
    if (BWD && i <= G.nx && j <= G.ny) {
        const int o = (j - 1 + HY) * G.pitch + (i - 1 + HX);
        bwd_conv<1>(G, F, M, W.sxx, W.syy, W.sxy, i, j, o, 0);
    }
}

// The stress update with VW adjacent cells per thread (VW = 2 or 4), the
// counterpart of k_update_vw: velocity stencils from 2K+1 vectors of a row
// (x) and one vector per row (y), model, memory variables and stresses as
// vectors; per cell the arithmetic of k_update_s, term by term. Reads past
// column NX + ND feed only cells past NX, which are never stored.
// The velocity derivatives of VW adjacent cells for the stress update
// (op_s_fdN, initfd.c:9-95, times 1/DH): ld(f, dy, dx, out) loads VW values
// of vx (f = 0) or vy (f = 1) at row j + dy, columns i + dx .. i + dx + VW - 1,
// from global memory in the stress kernels, from shared memory in the fused
// step kernel.
template <int ND, int VW, class LD>
__device__ __forceinline__ void s_derivs(const Geo &G, LD ld, float *vxx, float *vyx, float *vxy, float *vyy)
{
    constexpr int K = (ND + VW - 1) / VW;
    constexpr int NXS = VW * (2 * K + 1);
    const float *hc = G.hc;
    {
        float X[NXS], Y[NXS];  // X[k] = vx(j, i - VW K + k), Y[k] = vy(j, i - VW K + k)
#pragma unroll
        for (int q = 0; q < 2 * K + 1; q++) {
            ld(0, 0, VW * (q - K), X + VW * q);
            ld(1, 0, VW * (q - K), Y + VW * q);
        }
        constexpr int C = VW * K;
#pragma unroll
        for (int c = 0; c < VW; c++) {
            vxx[c] = hc[1] * (X[C + c] - X[C + c - 1]);
            vyx[c] = hc[1] * (Y[C + c + 1] - Y[C + c]);
#pragma unroll
            for (int m = 2; m <= ND; m++) {
                vxx[c] += hc[m] * (X[C + c + m - 1] - X[C + c - m]);
                vyx[c] += hc[m] * (Y[C + c + m] - Y[C + c - m + 1]);
            }
        }
    }
    {
        // y stencils: vx rows j - ND + 1 .. j + ND, vy rows j - ND .. j + ND - 1
        float a1[VW], a0[VW], b1[VW], b0[VW];
        ld(0, 1, 0, a1), ld(0, 0, 0, a0);
        ld(1, 0, 0, b1), ld(1, -1, 0, b0);
#pragma unroll
        for (int c = 0; c < VW; c++) {
            vxy[c] = hc[1] * (a1[c] - a0[c]);
            vyy[c] = hc[1] * (b1[c] - b0[c]);
        }
#pragma unroll
        for (int m = 2; m <= ND; m++) {
            ld(0, m, 0, a1), ld(0, -(m - 1), 0, a0);
            ld(1, m - 1, 0, b1), ld(1, -m, 0, b0);
#pragma unroll
            for (int c = 0; c < VW; c++) {
                vxy[c] += hc[m] * (a1[c] - a0[c]);
                vyy[c] += hc[m] * (b1[c] - b0[c]);
            }
        }
#pragma unroll
        for (int c = 0; c < VW; c++)
            vxx[c] *= G.dhi, vyx[c] *= G.dhi, vxy[c] *= G.dhi, vyy[c] *= G.dhi;
    }
}

// The stress and memory-variable update of VW adjacent cells (columns
// i .. i+VW-1, row j, padded offset o) from their velocity derivatives: CPML
// of the derivatives, isotropic / VTI stresses, L memory variables, damping
// frame; old stresses from Wr, new ones to Ww (the same arrays except in the
// fused step kernel), memory variables and CPML memory in place.
template <int ND, int KIND, bool VISCO, int LT, int VW, bool FWI = false>
__device__ __forceinline__ void s_update(const Geo &G, const Wave &Wr, const Wave &Ww, const Model &M, int s, int i,
                                         int j, int o, long long mo, float *vxx, float *vyx, float *vxy, float *vyy)
{
    const long long so = (long long)s * G.fsz;
    // old and new stresses are the same arrays outside the fused step kernel: no restrict here
    const float *sxx_o = Wr.sxx + so, *syy_o = Wr.syy + so, *sxy_o = Wr.sxy + so;
    float *sxx = Ww.sxx + so, *syy = Ww.syy + so, *sxy = Ww.sxy + so;
    const Wave &W = Wr;
    float m0[VW], m1[VW], m2[VW], m3[VW], b0[VW], b1[VW], b2[VW], b3[VW];
#pragma unroll
    for (int c = 0; c < VW; c++)
        m3[c] = 0.f, b0[c] = b1[c] = b2[c] = b3[c] = 0.f;
    if (KIND == ISO) {
        ldv<VW>(M.g + mo + o, m0), ldv<VW>(M.f + mo + o, m1), ldv<VW>(M.fipjp + mo + o, m2);
        if (VISCO)
            ldv<VW>(M.db + mo + o, b0), ldv<VW>(M.eb + mo + o, b1), ldv<VW>(M.dipb + mo + o, b2);
    } else {
        ldv<VW>(M.c11 + mo + o, m0), ldv<VW>(M.c13 + mo + o, m1), ldv<VW>(M.c33 + mo + o, m2);
        ldv<VW>(M.c55ipjp + mo + o, m3);
        if (VISCO) {
            ldv<VW>(M.c11b + mo + o, b0), ldv<VW>(M.c13b + mo + o, b1), ldv<VW>(M.c33b + mo + o, b2);
            ldv<VW>(M.c55ipjpb + mo + o, b3);
        }
    }
    constexpr int LN = LT > 0 ? LT : MAXL;
    const int L = LT > 0 ? LT : G.L;
    float *__restrict__ wr = W.r + (long long)s * G.L * G.fsz;
    float *__restrict__ wp = W.p + (long long)s * G.L * G.fsz;
    float *__restrict__ wq = W.q + (long long)s * G.L * G.fsz;
    float rr[LN][VW], pp[LN][VW], qq[LN][VW];
    if (VISCO) {
#pragma unroll
        for (int l = 0; l < LN; l++)
            if (l < L) {
                const long long lo = (long long)l * G.fsz + o;
                ldv_rw<VW>(wr + lo, rr[l]), ldv_rw<VW>(wp + lo, pp[l]), ldv_rw<VW>(wq + lo, qq[l]);
            }
    }
    float oxx[VW], oyy[VW], oxy[VW];
    ldv_rw<VW>(sxx_o + o, oxx), ldv_rw<VW>(syy_o + o, oyy), ldv_rw<VW>(sxy_o + o, oxy);
    const int yr = yside(G, j);
    const bool xframe = i <= G.gx2 || i + VW - 1 > G.gx3;
    float nxx[VW], nyy[VW], nxy[VW];
#pragma unroll
    for (int c = 0; c < VW; c++) {
        const int ic = i + c;
        const int xr = xframe ? xside(G, ic) : 0;
        float dxx = vxx[c], dyx = vyx[c], dxy = vxy[c], dyy = vyy[c];
        if (G.abs_type == 1 && ic <= G.nx)
            cpml_s(G, W, M, s, ic, j, xr, yr, dxx, dyx, dxy, dyy, true);
        float u1, u2, u3;
        if (KIND == ISO) {
            u1 = m2[c] * (dyx + dxy);
            float gd = m0[c] * (dxx + dyy);
            u2 = gd - 2.0f * m1[c] * dyy;
            u3 = gd - 2.0f * m1[c] * dxx;
            if (FWI && !VISCO && W.fstore && ic <= G.nx) {
                const long long n = (long long)G.nx * G.ny;
                float *slot = W.fstore + (long long)(*G.step_ctr - 1 - *W.fbase) * 5 * n +
                              ((long long)(j - 1) * G.nx + (ic - 1));
                slot[0] = W.fa_x[(long long)s * G.fsz + o + c], slot[n] = W.fa_y[(long long)s * G.fsz + o + c];
                slot[2 * n] = u2 / G.dt, slot[3 * n] = u3 / G.dt, slot[4 * n] = u1 / G.dt;
            }
        } else {
            u1 = m3[c] * (dxy + dyx);
            u2 = m0[c] * dxx + m1[c] * dyy;
            u3 = m1[c] * dxx + m2[c] * dyy;
        }
        if (VISCO) {
            float sro = 0.f, spo = 0.f, sqo = 0.f, sr = 0.f, sp = 0.f, sq = 0.f;
#pragma unroll
            for (int l = 0; l < LN; l++) {
                if (l < L) {
                    float r = rr[l][c], p = pp[l][c], q = qq[l][c];
                    sro += r, spo += p, sqo += q;
                    float pe = M.peta[l], bb = M.bip[l], cc = M.cip[l];
                    if (KIND == ISO) {
                        float dip = b2[c] * pe, d = b0[c] * pe, e = b1[c] * pe;
                        r = bb * (r * cc - dip * (dxy + dyx));
                        p = bb * (p * cc - e * (dxx + dyy) + 2.0f * d * dyy);
                        q = bb * (q * cc - e * (dxx + dyy) + 2.0f * d * dxx);
                    } else {
                        r = bb * (r * cc - (b3[c] * pe) * (dxy + dyx));
                        p = bb * (p * cc - (b0[c] * pe) * dxx - (b1[c] * pe) * dyy);
                        q = bb * (q * cc - (b1[c] * pe) * dxx - (b2[c] * pe) * dyy);
                    }
                    rr[l][c] = r, pp[l][c] = p, qq[l][c] = q;
                    sr += r, sp += p, sq += q;
                }
            }
            u1 += G.dthalbe * (sro + sr);
            u2 += G.dthalbe * (spo + sp);
            u3 += G.dthalbe * (sqo + sq);
        }
        nxy[c] = oxy[c] + u1, nxx[c] = oxx[c] + u2, nyy[c] = oyy[c] + u3;
        if (G.abs_type == 2 && (xr | yr)) {
            float a = __ldg(M.absorb + mo + o + c);
            nxy[c] *= a, nyy[c] *= a, nxx[c] *= a;
        }
    }
    if (i + VW - 1 <= G.nx) {
        if (VISCO) {
#pragma unroll
            for (int l = 0; l < LN; l++)
                if (l < L) {
                    const long long lo = (long long)l * G.fsz + o;
                    stv<VW>(wr + lo, rr[l]), stv<VW>(wp + lo, pp[l]), stv<VW>(wq + lo, qq[l]);
                }
        }
        stv<VW>(sxy + o, nxy), stv<VW>(sxx + o, nxx), stv<VW>(syy + o, nyy);
    } else {
#pragma unroll
        for (int c = 0; c < VW; c++) {
            if (i + c > G.nx)
                continue;
            if (VISCO) {
#pragma unroll
                for (int l = 0; l < LN; l++)
                    if (l < L) {
                        const long long lo = (long long)l * G.fsz + o + c;
                        wr[lo] = rr[l][c], wp[lo] = pp[l][c], wq[lo] = qq[l][c];
                    }
            }
            sxy[o + c] = nxy[c], sxx[o + c] = nxx[c], syy[o + c] = nyy[c];
        }
    }
}

template <int ND, int KIND, bool VISCO, int LT, int VW, bool FWI = false, int TBX = BX, bool BWD = false>
__device__ __forceinline__ void sw_tile(const Geo &G, const Wave &W, const Model &M, const uint3 b,
                                        const FwiDev *F = nullptr)
{
    constexpr int TBY = BX * BY / TBX;  // TBX: as in vw_tile
    int bx, s;
    block_xs(G, b, bx, s);
    const int i = (bx * TBX + threadIdx.x) * VW + 1;
    const int j = b.y * TBY + threadIdx.y + 1;
    // the step this kernel completes, for the next backward velocity kernel
    // (nothing writes the step counter while it runs)
    if (BWD && b.x == 0 && b.y == 0 && b.z == 0 && threadIdx.x == 0 && threadIdx.y == 0)
        *F->bstep = *G.step_ctr;
    if (i > G.nx || j > G.ny)
        return;
    const int P = G.pitch;
    const int o = (j - 1 + HY) * P + (i - 1 + HX);
    const long long so = (long long)s * G.fsz, mo = moff(G, s);
    const float *__restrict__ vx = W.vx + so;
    const float *__restrict__ vy = W.vy + so;
    float vxx[VW], vyx[VW], vxy[VW], vyy[VW];
    s_derivs<ND, VW>(
        G, [&](int f, int dy, int dx, float *out) { ldv<VW>((f ? vy : vx) + o + dy * P + dx, out); }, vxx, vyx,
        vxy, vyy);
    s_update<ND, KIND, VISCO, LT, VW, FWI>(G, W, W, M, s, i, j, o, mo, vxx, vyx, vxy, vyy);
    if constexpr (BWD)
        bwd_conv<VW>(G, *F, M, W.sxx + so, W.syy + so, W.sxy + so, i, j, o, mo);
}

template <int ND, int KIND, bool VISCO, int LT, int VW, bool FWI = false, int TBX = BX>
__global__ void __launch_bounds__(BX *BY, VW == 4 ? (VISCO ? 2 : 3) : 1) k_update_sw(Geo G, Wave W, Model M)
{
    pdl_begin();
    sw_tile<ND, KIND, VISCO, LT, VW, FWI, TBX>(G, W, M, blockIdx);
}

// A backward step of an FWI pass (EL_ISO) without a free surface: the
// elastic stress update of VW = 4, 2 or 1 cells per thread, then the lambda /
// mu correlation (bwd_conv) in the same kernel.
template <int ND, int VW>
__global__ void __launch_bounds__(BX *BY, VW == 4 ? 2 : 1) k_update_sw_bwd(Geo G, Wave W, Model M, FwiDev F)
{
    pdl_begin();
    sw_tile<ND, ISO, false, 0, VW, false, BX, true>(G, W, M, blockIdx, &F);
}

// Acoustic stress update (wavefield_update_s_ac.c, update_s_acoustic_{interior,
// PML,abs}.c), VW cells per thread (1, 2 or 4). The reference allocates one
// array for sxx and syy (initmem_wavefield.c:34), so the pressure p = sxx = syy
// gets g*vxx and then g*vyy, rounded in that order; the velocity update reads
// the same array for its x and y derivatives. CPML stretches vxx in the left /
// right frame and vyy in the top / bottom frame (cpml_update_s_x_ac,
// cpml_update_s_y_ac); the damping frame multiplies p once (abs_update_s_ac2).
template <int ND, int VW>
__device__ __forceinline__ void sac_tile(const Geo &G, const Wave &W, const Model &M, const uint3 b)
{
    constexpr int K = (ND + VW - 1) / VW;
    constexpr int NXS = VW * (2 * K + 1);
    int bx, s;
    block_xs(G, b, bx, s);
    const int i = (bx * BX + threadIdx.x) * VW + 1;
    const int j = b.y * BY + threadIdx.y + 1;
    if (i > G.nx || j > G.ny)
        return;
    const int P = G.pitch;
    const int o = (j - 1 + HY) * P + (i - 1 + HX);
    const long long so = (long long)s * G.fsz, mo = moff(G, s);
    float *__restrict__ pr = W.sxx + so;
    const float *__restrict__ vx = W.vx + so;
    const float *__restrict__ vy = W.vy + so;
    const float *hc = G.hc;
    float vxx[VW], vyy[VW];
    {
        float X[NXS];  // X[k] = vx(j, i - VW K + k)
#pragma unroll
        for (int q = 0; q < 2 * K + 1; q++)
            ldv<VW>(vx + o + VW * (q - K), X + VW * q);
        constexpr int C = VW * K;
#pragma unroll
        for (int c = 0; c < VW; c++) {
            vxx[c] = hc[1] * (X[C + c] - X[C + c - 1]);
#pragma unroll
            for (int m = 2; m <= ND; m++)
                vxx[c] += hc[m] * (X[C + c + m - 1] - X[C + c - m]);
        }
    }
    {
        float b1[VW], b0[VW];  // vy rows j - ND .. j + ND - 1
        ldv<VW>(vy + o, b1), ldv<VW>(vy + o - P, b0);
#pragma unroll
        for (int c = 0; c < VW; c++)
            vyy[c] = hc[1] * (b1[c] - b0[c]);
#pragma unroll
        for (int m = 2; m <= ND; m++) {
            ldv<VW>(vy + o + (m - 1) * P, b1), ldv<VW>(vy + o - m * P, b0);
#pragma unroll
            for (int c = 0; c < VW; c++)
                vyy[c] += hc[m] * (b1[c] - b0[c]);
        }
#pragma unroll
        for (int c = 0; c < VW; c++)
            vxx[c] *= G.dhi, vyy[c] *= G.dhi;
    }
    float g[VW], op[VW], np[VW];
    ldv<VW>(M.g + mo + o, g);
    ldv_rw<VW>(pr + o, op);
    const int yr = yside(G, j);
    const bool xframe = i <= G.gx2 || i + VW - 1 > G.gx3;
#pragma unroll
    for (int c = 0; c < VW; c++) {
        const int ic = i + c;
        const int xr = xframe ? xside(G, ic) : 0;
        float dxx = vxx[c], dyy = vyy[c];
        if (G.abs_type == 1 && ic <= G.nx) {
            if (xr) {
                const int h = xr == 1 ? ic : ic - G.nx + G.fw2;
                const long long q = ((long long)s * G.ny + (j - 1)) * G.fw2 + (h - 1);
                const float ps = M.b_x[h - 1] * W.psi_vxx[q] + M.a_x[h - 1] * dxx;
                W.psi_vxx[q] = ps;
                dxx = dxx / M.K_x[h - 1] + ps;
            }
            if (yr) {
                const int h = yr == 1 ? j : j - G.ny + G.fw2;
                const long long q = ((long long)s * G.fw2 + (h - 1)) * G.nx + (ic - 1);
                const float ps = M.b_y[h - 1] * W.psi_vyy[q] + M.a_y[h - 1] * dyy;
                W.psi_vyy[q] = ps;
                dyy = dyy / M.K_y[h - 1] + ps;
            }
        }
        float t = op[c] + g[c] * dxx;
        t = t + g[c] * dyy;
        if (G.abs_type == 2 && (xr | yr))
            t *= __ldg(M.absorb + mo + o + c);
        np[c] = t;
    }
    if (i + VW - 1 <= G.nx) {
        stv<VW>(pr + o, np);
    } else {
#pragma unroll
        for (int c = 0; c < VW; c++)
            if (i + c <= G.nx)
                pr[o + c] = np[c];
    }
}

template <int ND, int VW>
__global__ void __launch_bounds__(BX *BY) k_update_s_ac(Geo G, Wave W, Model M)
{
    pdl_begin();
    sac_tile<ND, VW>(G, W, M, blockIdx);
}

// ------------------------------------------------------------------ TTI

// Raw velocity derivatives of every cell and their CPML-stretched values
// (equal to the raw ones outside the CPML passes); updates psi_v.
template <int ND>
__global__ void __launch_bounds__(BX *BY) k_tti_deriv(Geo G, Wave W, Model M)
{
    int bx, s;
    block_xs(G, bx, s);
    int i = bx * BX + threadIdx.x + 1;
    int j = blockIdx.y * BY + threadIdx.y + 1;
    if (i > G.nx || j > G.ny)
        return;
    long long o = cell(G, j, i);
    long long so = (long long)s * G.fsz;
    float vxx, vyx, vxy, vyy;
    op_s<ND>(W.vx + so, W.vy + so, o, G.pitch, G.hc, G.dhi, vxx, vyx, vxy, vyy);
    float *dr = W.draw + 4 * so, *dc = W.dcor + 4 * so;
    dr[o] = vxx, dr[G.fsz + o] = vyy, dr[2 * G.fsz + o] = vyx, dr[3 * G.fsz + o] = vxy;
    if (G.abs_type == 1) {
        int xr = xside(G, i), yr = yside(G, j);
        bool skip = G.el_tti_rb_short && xr == 2 && yr == 2 && j == G.ny;
        if (!skip)
            cpml_s(G, W, M, s, i, j, xr, yr, vxx, vyx, vxy, vyy, true);
    }
    dc[o] = vxx, dc[G.fsz + o] = vyy, dc[2 * G.fsz + o] = vyx, dc[3 * G.fsz + o] = vxy;
}

// Derivative k (0 vxx, 1 vyy, 2 vyx, 3 vxy) of neighbour (jn, in) as the
// reference's TTI update of a cell in region rc sees it: stretched if the
// neighbour's region had its CPML pass before rc's update pass (regions are
// processed in order, the interior first, each region's CPML pass before its
// update pass), raw otherwise; zero outside the grid (periodic x: the raw
// value of the wrapped column, copied before any stretch).
__device__ __forceinline__ float tti_d(const Geo &G, const float *dr, const float *dc, int k, int jn, int in,
                                       int rc)
{
    if (jn < 1 || jn > G.ny)
        return 0.f;
    if (in < 1 || in > G.nx) {
        if (!G.boundary)
            return 0.f;
        in = in < 1 ? in + G.nx : in - G.nx;
        return dr[k * G.fsz + cell(G, jn, in)];
    }
    long long o = cell(G, jn, in);
    int rn = region(G, in, jn);
    return (rn <= rc) ? dc[k * G.fsz + o] : dr[k * G.fsz + o];
}

// The stress / memory-variable arithmetic of wavefield_update_s_el_tti.c:27-52 and
// wavefield_update_s_visc_TTI.c:27-84 for cell o, given the derivatives at the
// cell and the 4-point averages the reference forms from its neighbours.
template <bool VISCO>
__device__ __forceinline__ void tti_update(const Geo &G, const Wave &W, const Model &M, int s, long long o, int xr,
                                           int yr, float vxx, float vyy, float vxxipjp, float vyyipjp, float vyx0,
                                           float vxy0, float vyxij, float vxyij)
{
    const long long so = (long long)s * G.fsz, mo = moff(G, s);
    float vij = vyxij + vxyij;
    float v = vxy0 + vyx0;
    float u1 = __ldg(M.c55ipjp + mo + o) * v + __ldg(M.c15ipjp + mo + o) * vxxipjp +
               __ldg(M.c35ipjp + mo + o) * vyyipjp;
    float u2 = __ldg(M.c11 + mo + o) * vxx + __ldg(M.c13 + mo + o) * vyy + __ldg(M.c15 + mo + o) * vij;
    float u3 = __ldg(M.c13 + mo + o) * vxx + __ldg(M.c33 + mo + o) * vyy + __ldg(M.c35 + mo + o) * vij;
    if (VISCO) {
        float b55 = __ldg(M.c55ipjpb + mo + o), b15i = __ldg(M.c15ipjpb + mo + o), b35i = __ldg(M.c35ipjpb + mo + o);
        float b11 = __ldg(M.c11b + mo + o), b13 = __ldg(M.c13b + mo + o), b33 = __ldg(M.c33b + mo + o);
        float b15 = __ldg(M.c15b + mo + o), b35 = __ldg(M.c35b + mo + o);
        float sro = 0.f, spo = 0.f, sqo = 0.f, sr = 0.f, sp = 0.f, sq = 0.f;
        for (int l = 0; l < G.L; l++) {
            long long lo = ((long long)s * G.L + l) * G.fsz + o;
            float r = W.r[lo], p = W.p[lo], q = W.q[lo];
            sro += r, spo += p, sqo += q;
            float pe = M.peta[l], b = M.bip[l], c = M.cip[l];
            r = b * (r * c - (b55 * pe) * v - (b15i * pe) * vxxipjp - (b35i * pe) * vyyipjp);
            p = b * (p * c - (b11 * pe) * vxx - (b13 * pe) * vyy - (b15 * pe) * vij);
            q = b * (q * c - (b13 * pe) * vxx - (b33 * pe) * vyy - (b35 * pe) * vij);
            W.r[lo] = r, W.p[lo] = p, W.q[lo] = q;
            sr += r, sp += p, sq += q;
        }
        u1 += G.dthalbe * (sro + sr);
        u2 += G.dthalbe * (spo + sp);
        u3 += G.dthalbe * (sqo + sq);
    }
    float nxy = W.sxy[so + o] + u1, nxx = W.sxx[so + o] + u2, nyy = W.syy[so + o] + u3;
    if (G.abs_type == 2 && (xr | yr)) {
        float a = __ldg(M.absorb + mo + o);
        nxy *= a, nyy *= a, nxx *= a;
    }
    W.sxy[so + o] = nxy;
    W.sxx[so + o] = nxx;
    W.syy[so + o] = nyy;
}

// TTI CPML driver: cells the reference's update_s_*_TTI_PML.c loops skip
// (two outer cells of each frame side, update_s_elastic_TTI_PML.c:44,58,69,82).
__device__ __forceinline__ bool tti_pml_skipped(const Geo &G, int i, int j, int xr, int yr)
{
    return G.abs_type == 1 &&
           ((xr == 1 && i < 3) || (xr == 2 && i > G.nx - 2) || (yr == 1 && j < 3) || (yr == 2 && j > G.ny - 2));
}

// The stress update from the derivative fields k_tti_deriv stored.
template <bool VISCO>
__global__ void __launch_bounds__(BX *BY) k_update_s_tti(Geo G, Wave W, Model M)
{
    int bx, s;
    block_xs(G, bx, s);
    int i = bx * BX + threadIdx.x + 1;
    int j = blockIdx.y * BY + threadIdx.y + 1;
    if (i > G.nx || j > G.ny)
        return;
    int xr = xside(G, i), yr = yside(G, j);
    if (tti_pml_skipped(G, i, j, xr, yr))
        return;
    long long o = cell(G, j, i);
    long long so = (long long)s * G.fsz;
    const float *dr = W.draw + 4 * so, *dc = W.dcor + 4 * so;
    int rc = (G.abs_type == 1) ? region(G, i, j) : 0;
    float vxx = tti_d(G, dr, dc, 0, j, i, rc), vyy = tti_d(G, dr, dc, 1, j, i, rc);
    float vxxipjp = 0.25f * (vxx + tti_d(G, dr, dc, 0, j + 1, i, rc) + tti_d(G, dr, dc, 0, j, i + 1, rc) +
                             tti_d(G, dr, dc, 0, j + 1, i + 1, rc));
    float vyyipjp = 0.25f * (vyy + tti_d(G, dr, dc, 1, j + 1, i, rc) + tti_d(G, dr, dc, 1, j, i + 1, rc) +
                             tti_d(G, dr, dc, 1, j + 1, i + 1, rc));
    float vyx0 = tti_d(G, dr, dc, 2, j, i, rc), vxy0 = tti_d(G, dr, dc, 3, j, i, rc);
    float vyxij = 0.25f * (vyx0 + tti_d(G, dr, dc, 2, j - 1, i, rc) + tti_d(G, dr, dc, 2, j, i - 1, rc) +
                           tti_d(G, dr, dc, 2, j - 1, i - 1, rc));
    float vxyij = 0.25f * (vxy0 + tti_d(G, dr, dc, 3, j - 1, i, rc) + tti_d(G, dr, dc, 3, j, i - 1, rc) +
                           tti_d(G, dr, dc, 3, j - 1, i - 1, rc));
    tti_update<VISCO>(G, W, M, s, o, xr, yr, vxx, vyy, vxxipjp, vyyipjp, vyx0, vxy0, vyxij, vxyij);
}

// The whole TTI stress half-step in one pass. A block derives the four velocity
// derivatives of its 32 x 8 tile and of the one-cell ring around it (the cells
// the 4-point averages reach) into shared memory, raw and CPML-stretched, then
// updates its tile. A neighbour's derivative is taken stretched or raw by the
// reference's region order, as tti_d does. Ring cells belong to other blocks,
// which write their CPML memory: every block reads the memory of the previous
// step's buffer and only the owner of a cell writes this step's buffer
// (Geo::psi_pp), so no block sees a value another block has already advanced.
// tti_tile: the tile with origin (i0, j0) of shot s, thread (tx, ty) of the
// 32 x 8 block, sd: NB [4][BY + 2][BX + 2] arrays of shared memory; cells in
// [ki0, ki1] x [kj0, kj1] are left to another block (their derivatives still
// feed this tile's averages).
template <int ND, bool VISCO, bool CPML>
__device__ __forceinline__ void tti_tile(const Geo &G, const Wave &W, const Model &M, int s, int i0, int j0, int tx,
                                         int ty, float (*sd)[4][BY + 2][BX + 2], int ki0 = 1, int ki1 = 0,
                                         int kj0 = 1, int kj1 = 0)
{
    constexpr int SX = BX + 2, SY = BY + 2, NB = CPML ? 2 : 1;
    constexpr int RING = 2 * SX + 2 * BY;
    static_assert(RING <= BX * BY, "ring cells exceed the block");
    const int tid = ty * BX + tx;
    const long long so = (long long)s * G.fsz;
    const float *vx = W.vx + so, *vy = W.vy + so;
    Wave Wn = W, Wo = W;
    if (CPML) {
        psi_buffers(G, Wn, false);
        psi_buffers(G, Wo, true);
    }
    // tile and ring wholly inside the interior region: no stretch, one region,
    // raw and stretched derivatives coincide (block-uniform)
    const bool frame = CPML && !(i0 - 1 > G.gx2 && i0 + BX <= G.gx3 && j0 - 1 > G.gy2 && j0 + BY <= G.gy3);
    // pass 0: the tile (one cell per thread); pass 1: the ring (first RING threads)
#pragma unroll 1
    for (int pass = 0; pass < 2; pass++) {
        int ly, lx;
        if (pass == 0) {
            ly = ty + 1, lx = tx + 1;
        } else {
            if (tid >= RING)
                break;
            if (tid < SX) {
                ly = 0, lx = tid;
            } else if (tid < 2 * SX) {
                ly = SY - 1, lx = tid - SX;
            } else {
                const int t = tid - 2 * SX;
                ly = 1 + (t >> 1), lx = (t & 1) ? SX - 1 : 0;
            }
        }
        const int jn = j0 - 1 + ly, in = i0 - 1 + lx;
        float d[4] = {0.f, 0.f, 0.f, 0.f};
        float c[4];
        int ic = 0;  // column the derivatives are taken at (0: none, zero)
        if (jn >= 1 && jn <= G.ny) {
            if (in >= 1 && in <= G.nx)
                ic = in;
            else if (G.boundary) {
                ic = in < 1 ? in + G.nx : in - G.nx;  // periodic x: the wrapped column, raw
                if (ic < 1 || ic > G.nx)              // past the ring no cell reads (grids < 32 wide)
                    ic = 0;
            }
        }
        if (ic)
            op_s<ND>(vx, vy, cell(G, jn, ic), G.pitch, G.hc, G.dhi, d[0], d[2], d[3], d[1]);
#pragma unroll
        for (int k = 0; k < 4; k++)
            c[k] = d[k];
        if (frame && ic && ic == in) {
            const int xr = xside(G, in), yr = yside(G, jn);
            if (xr | yr) {
                const bool own = pass == 0;
                if (!(G.el_tti_rb_short && xr == 2 && yr == 2 && jn == G.ny)) {
                    cpml_s2(G, Wo, Wn, M, s, in, jn, xr, yr, c[0], c[2], c[3], c[1], own);
                } else if (own) {
                    // the reference's right-bottom pass stops at NY-1: memory unchanged
                    const int hx = in - G.nx + G.fw2, hy = jn - G.ny + G.fw2;
                    const long long qx = ((long long)s * G.ny + (jn - 1)) * G.fw2 + (hx - 1);
                    const long long qy = ((long long)s * G.fw2 + (hy - 1)) * G.nx + (in - 1);
                    Wn.psi_vxx[qx] = Wo.psi_vxx[qx], Wn.psi_vyx[qx] = Wo.psi_vyx[qx];
                    Wn.psi_vyy[qy] = Wo.psi_vyy[qy], Wn.psi_vxy[qy] = Wo.psi_vxy[qy];
                }
            }
        }
#pragma unroll
        for (int k = 0; k < 4; k++) {
            sd[0][k][ly][lx] = d[k];
            if (frame)
                sd[NB - 1][k][ly][lx] = c[k];
        }
    }
    __syncthreads();
    const int i = i0 + tx, j = j0 + ty;
    if (i > G.nx || j > G.ny || (i >= ki0 && i <= ki1 && j >= kj0 && j <= kj1))
        return;
    const int xr = xside(G, i), yr = yside(G, j);
    if (tti_pml_skipped(G, i, j, xr, yr))
        return;
    const int rc = frame ? region(G, i, j) : 0;
    const int sy = ty + 1, sx = tx + 1;
    // derivative k of neighbour (j + dy, i + dx) as the update of this cell sees it
    auto D = [&](int k, int dy, int dx) -> float {
        if (!frame)
            return sd[0][k][sy + dy][sx + dx];
        const int jn = j + dy, in = i + dx;
        if (jn < 1 || jn > G.ny || in < 1 || in > G.nx)
            return sd[0][k][sy + dy][sx + dx];
        return region(G, in, jn) <= rc ? sd[NB - 1][k][sy + dy][sx + dx] : sd[0][k][sy + dy][sx + dx];
    };
    const float vxx = D(0, 0, 0), vyy = D(1, 0, 0);
    const float vxxipjp = 0.25f * (vxx + D(0, 1, 0) + D(0, 0, 1) + D(0, 1, 1));
    const float vyyipjp = 0.25f * (vyy + D(1, 1, 0) + D(1, 0, 1) + D(1, 1, 1));
    const float vyx0 = D(2, 0, 0), vxy0 = D(3, 0, 0);
    const float vyxij = 0.25f * (vyx0 + D(2, -1, 0) + D(2, 0, -1) + D(2, -1, -1));
    const float vxyij = 0.25f * (vxy0 + D(3, -1, 0) + D(3, 0, -1) + D(3, -1, -1));
    tti_update<VISCO>(G, W, M, s, cell(G, j, i), xr, yr, vxx, vyy, vxxipjp, vyyipjp, vyx0, vxy0, vyxij, vxyij);
}

template <int ND, bool VISCO, bool CPML>
__global__ void __launch_bounds__(BX *BY) k_tti_fused(Geo G, Wave W, Model M)
{
    __shared__ float sd[CPML ? 2 : 1][4][BY + 2][BX + 2];  // [raw, stretched][vxx vyy vyx vxy][y][x]
    pdl_begin();
    int bx, s;
    block_xs(G, bx, s);
    tti_tile<ND, VISCO, CPML>(G, W, M, s, bx * BX + 1, blockIdx.y * BY + 1, threadIdx.x, threadIdx.y, sd);
}

// The TTI stress update over two kinds of tile in one launch. The interior
// rectangle [fi0, fi1] x [fj0, fj1] holds the cells whose one-cell ring lies
// inside the grid and inside the CPML (or damping) frame's interior (every
// cell and neighbour in region 0: no stretch, no damping); its width is a
// multiple of 4 and fi0 - 1 a multiple of 4 (16-byte aligned rows). It is cut
// into tiles of up to 64 x 32 cells (origin (fi0 + 64 a, fj0 + 32 b)) that
// take tti_tile4. The 32 x 8 tiles of the grid not wholly inside the
// rectangle take tti_tile, the one-pass form above, and skip the cells that
// lie inside it. The frame's tiles come first in the launch, so their longer
// blocks start before the bulk of the interior ones.
struct TtiMap {
    int nsx, nsy;              // 32 x 8 tiles of the grid, per row and column
    int sxa, sxb, sya, syb;    // the 32 x 8 tiles wholly inside the rectangle (inclusive; none: sya = nsy)
    int nframe;                // 32 x 8 tiles outside that range: blocks 0 .. nframe - 1
    int fi0, fi1, fj0, fj1;    // the interior rectangle (empty: fi1 < fi0)
    int nfx, nfy;              // its tiles: blocks nframe + b * nfx + a, a < nfx, b < nfy
};
constexpr int T4X = 64, T4Y = 32;       // cells of an interior tile
constexpr int T4W = 72, T4P = 34 * 72;  // shared row (column 3: i0 - 1, 4 ..: the tile, 68: i0 + 64), plane

// 32 x 8 tile (sx, sy) of frame block b: the rows above the 64 x 32 tiles,
// then per row of theirs the tiles left and right of them, then the rows below.
__device__ __forceinline__ void tti_frame_tile(const TtiMap &T, int b, int &sx, int &sy)
{
    const int top = T.sya * T.nsx;
    if (b < top) {
        sy = b / T.nsx, sx = b - sy * T.nsx;
        return;
    }
    b -= top;
    const int side = T.sxa + (T.nsx - 1 - T.sxb), mid = (T.syb - T.sya + 1) * side;
    if (b < mid) {
        const int r = b / side, k = b - r * side;
        sy = T.sya + r, sx = k < T.sxa ? k : T.sxb + 1 + (k - T.sxa);
        return;
    }
    b -= mid;
    const int r = b / T.nsx;
    sy = T.syb + 1 + r, sx = b - r * T.nsx;
}

__device__ __forceinline__ void lds4(const float *p, float *out)
{
    const float4 a = *reinterpret_cast<const float4 *>(p);
    out[0] = a.x, out[1] = a.y, out[2] = a.z, out[3] = a.w;
}

// tti_update for the four cells o .. o + 3 of one row (interior: no damping),
// model, memory variables and stresses as 16-byte vectors; per cell the
// expressions of tti_update, term by term.
template <bool VISCO>
__device__ __forceinline__ void tti_update4(const Geo &G, const Wave &W, const Model &M, int s, int o, long long mo,
                                            const float *vxx, const float *vyy, const float *vxxipjp,
                                            const float *vyyipjp, const float *vyx0, const float *vxy0,
                                            const float *vyxij, const float *vxyij)
{
    const long long so = (long long)s * G.fsz;
    float u1[4], u2[4], u3[4];
    {
        float a[4], b[4], c[4];
        ldv_once<4>(M.c55ipjp + mo + o, a), ldv_once<4>(M.c15ipjp + mo + o, b), ldv_once<4>(M.c35ipjp + mo + o, c);
#pragma unroll
        for (int k = 0; k < 4; k++)
            u1[k] = a[k] * (vxy0[k] + vyx0[k]) + b[k] * vxxipjp[k] + c[k] * vyyipjp[k];
    }
    {
        float c11[4], c13[4], c33[4], c15[4], c35[4];
        ldv_once<4>(M.c11 + mo + o, c11), ldv_once<4>(M.c13 + mo + o, c13), ldv_once<4>(M.c33 + mo + o, c33);
        ldv_once<4>(M.c15 + mo + o, c15), ldv_once<4>(M.c35 + mo + o, c35);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const float vij = vyxij[k] + vxyij[k];
            u2[k] = c11[k] * vxx[k] + c13[k] * vyy[k] + c15[k] * vij;
            u3[k] = c13[k] * vxx[k] + c33[k] * vyy[k] + c35[k] * vij;
        }
    }
    if (VISCO) {
        float sro[4], spo[4], sqo[4], sr[4], sp[4], sq[4];
#pragma unroll
        for (int k = 0; k < 4; k++)
            sro[k] = spo[k] = sqo[k] = sr[k] = sp[k] = sq[k] = 0.f;
        for (int l = 0; l < G.L; l++) {
            const long long lo = ((long long)s * G.L + l) * G.fsz + o;
            const float pe = M.peta[l], bb = M.bip[l], cc = M.cip[l];
            float r[4], p[4], q[4], x[4], y[4], z[4];
            ldv_rw_once<4>(W.r + lo, r), ldv_rw_once<4>(W.p + lo, p), ldv_rw_once<4>(W.q + lo, q);
            ldv_once<4>(M.c55ipjpb + mo + o, x), ldv_once<4>(M.c15ipjpb + mo + o, y), ldv_once<4>(M.c35ipjpb + mo + o, z);
#pragma unroll
            for (int k = 0; k < 4; k++) {
                sro[k] += r[k];
                r[k] = bb * (r[k] * cc - (x[k] * pe) * (vxy0[k] + vyx0[k]) - (y[k] * pe) * vxxipjp[k] -
                             (z[k] * pe) * vyyipjp[k]);
                sr[k] += r[k];
            }
            stv<4>(W.r + lo, r);
            ldv_once<4>(M.c11b + mo + o, x), ldv_once<4>(M.c13b + mo + o, y), ldv_once<4>(M.c15b + mo + o, z);
#pragma unroll
            for (int k = 0; k < 4; k++) {
                spo[k] += p[k];
                p[k] = bb * (p[k] * cc - (x[k] * pe) * vxx[k] - (y[k] * pe) * vyy[k] -
                             (z[k] * pe) * (vyxij[k] + vxyij[k]));
                sp[k] += p[k];
            }
            stv<4>(W.p + lo, p);
            ldv_once<4>(M.c33b + mo + o, x), ldv_once<4>(M.c35b + mo + o, z);
#pragma unroll
            for (int k = 0; k < 4; k++) {
                sqo[k] += q[k];
                q[k] = bb * (q[k] * cc - (y[k] * pe) * vxx[k] - (x[k] * pe) * vyy[k] -
                             (z[k] * pe) * (vyxij[k] + vxyij[k]));
                sq[k] += q[k];
            }
            stv<4>(W.q + lo, q);
        }
#pragma unroll
        for (int k = 0; k < 4; k++) {
            u1[k] += G.dthalbe * (sro[k] + sr[k]);
            u2[k] += G.dthalbe * (spo[k] + sp[k]);
            u3[k] += G.dthalbe * (sqo[k] + sq[k]);
        }
    }
    float oxy[4], oxx[4], oyy[4];
    ldv_rw_once<4>(W.sxy + so + o, oxy), ldv_rw_once<4>(W.sxx + so + o, oxx), ldv_rw_once<4>(W.syy + so + o, oyy);
#pragma unroll
    for (int k = 0; k < 4; k++)
        oxy[k] += u1[k], oxx[k] += u2[k], oyy[k] += u3[k];
    stv<4>(W.sxy + so + o, oxy), stv<4>(W.sxx + so + o, oxx), stv<4>(W.syy + so + o, oyy);
}

// The velocity derivatives of the four-cell groups of rows j and j + 1
// (columns i .. i + 3, padded offset o of (j, i)), stored to shared memory at
// q (row j) and q + row (row j + 1), planes plane apart: vxx vyy vyx vxy. The
// y stencils of both rows come from one window of 2 ND + 1 rows of vx and of
// vy; per cell the expressions of s_derivs, term by term.
template <int ND>
__device__ __forceinline__ void s_derivs_pair(const Geo &G, const float *__restrict__ vx,
                                              const float *__restrict__ vy, int o, int P, float *q, int row,
                                              int plane)
{
    const float *hc = G.hc;
    constexpr int K = (ND + 3) / 4, NXS = 4 * (2 * K + 1), C = 4 * K;
#pragma unroll
    for (int h = 0; h < 2; h++) {  // x stencils, row by row
        float X[NXS], Y[NXS];
#pragma unroll
        for (int u = 0; u < 2 * K + 1; u++) {
            ldv<4>(vx + o + h * P + 4 * (u - K), X + 4 * u);
            ldv<4>(vy + o + h * P + 4 * (u - K), Y + 4 * u);
        }
        float dxx[4], dyx[4];
#pragma unroll
        for (int c = 0; c < 4; c++) {
            dxx[c] = hc[1] * (X[C + c] - X[C + c - 1]);
            dyx[c] = hc[1] * (Y[C + c + 1] - Y[C + c]);
#pragma unroll
            for (int m = 2; m <= ND; m++) {
                dxx[c] += hc[m] * (X[C + c + m - 1] - X[C + c - m]);
                dyx[c] += hc[m] * (Y[C + c + m] - Y[C + c - m + 1]);
            }
            dxx[c] *= G.dhi, dyx[c] *= G.dhi;
        }
        stv<4>(q + h * row, dxx), stv<4>(q + h * row + 2 * plane, dyx);
    }
    {
        // vx rows j - ND + 1 .. j + ND + 1: R[d] = vx(j - ND + 1 + d)
        float R[2 * ND + 1][4];
#pragma unroll
        for (int d = 0; d < 2 * ND + 1; d++)
            ldv<4>(vx + o + (d - ND + 1) * P, R[d]);
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int z = ND - 1 + h;  // index of row j + h
            float dxy[4];
#pragma unroll
            for (int c = 0; c < 4; c++) {
                dxy[c] = hc[1] * (R[z + 1][c] - R[z][c]);
#pragma unroll
                for (int m = 2; m <= ND; m++)
                    dxy[c] += hc[m] * (R[z + m][c] - R[z - (m - 1)][c]);
                dxy[c] *= G.dhi;
            }
            stv<4>(q + h * row + 3 * plane, dxy);
        }
    }
    {
        // vy rows j - ND .. j + ND: R[d] = vy(j - ND + d)
        float R[2 * ND + 1][4];
#pragma unroll
        for (int d = 0; d < 2 * ND + 1; d++)
            ldv<4>(vy + o + (d - ND) * P, R[d]);
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int z = ND + h;  // index of row j + h
            float dyy[4];
#pragma unroll
            for (int c = 0; c < 4; c++) {
                dyy[c] = hc[1] * (R[z][c] - R[z - 1][c]);
#pragma unroll
                for (int m = 2; m <= ND; m++)
                    dyy[c] += hc[m] * (R[z + m - 1][c] - R[z - m][c]);
                dyy[c] *= G.dhi;
            }
            stv<4>(q + h * row + plane, dyy);
        }
    }
}

// One interior tile with origin (i0, j0) of cols x rows cells (cols a multiple
// of 4, at most 64; rows at most 32), 256 threads: each thread derives four
// adjacent cells of two adjacent rows (16-byte loads, s_derivs_pair: one
// window of rows for both rows' y stencils), warps 0-3 derive the
// ring (the rows above and below as four-cell groups, the columns left and
// right cell by cell), all into sm ([vxx vyy vyx vxy][34][72]: row 0 is
// j0 - 1, column 3 is i0 - 1); then each thread updates its cells from there.
// No cell of the tile or its ring is in the frame, so raw and stretched
// derivatives coincide.
template <int ND, bool VISCO>
__device__ __forceinline__ void tti_tile4(const Geo &G, const Wave &W, const Model &M, int s, int i0, int j0,
                                          int cols, int rows, float *sm)
{
    const int t = threadIdx.x, gx = t & 15, gy = t >> 4, w = t >> 5, lane = t & 31;
    const int P = G.pitch;
    const long long so = (long long)s * G.fsz;
    const float *__restrict__ vx = W.vx + so;
    const float *__restrict__ vy = W.vy + so;
    // four-cell group at row j, columns i .. i + 3 -> shared row r, column x
    auto group = [&](int j, int i, int r, int x) {
        const int o = (j - 1 + HY) * P + (i - 1 + HX);
        float dxx[4], dyx[4], dxy[4], dyy[4];
        s_derivs<ND, 4>(
            G, [&](int f, int dy, int dx, float *out) { ldv<4>((f ? vy : vx) + o + dy * P + dx, out); }, dxx, dyx,
            dxy, dyy);
        float *q = sm + r * T4W + x;
        stv<4>(q, dxx), stv<4>(q + T4P, dyy), stv<4>(q + 2 * T4P, dyx), stv<4>(q + 3 * T4P, dxy);
    };
    // one cell (j, i) -> shared row r, column x
    auto single = [&](int j, int i, int r, int x) {
        float d0, d1, d2, d3;
        op_s<ND>(vx, vy, cell(G, j, i), P, G.hc, G.dhi, d0, d2, d3, d1);
        float *q = sm + r * T4W + x;
        q[0] = d0, q[T4P] = d1, q[2 * T4P] = d2, q[3 * T4P] = d3;
    };
    const bool gon = 4 * gx < cols;
    const int r0 = 2 * gy;  // this thread's rows: r0 and r0 + 1
    if (gon && r0 + 1 < rows)
        s_derivs_pair<ND>(G, vx, vy, (j0 + r0 - 1 + HY) * P + (i0 + 4 * gx - 1 + HX), P,
                          sm + (r0 + 1) * T4W + 4 + 4 * gx, T4W, T4P);
    else if (gon && r0 < rows)
        group(j0 + r0, i0 + 4 * gx, r0 + 1, 4 + 4 * gx);
    if (w == 0) {  // rows j0 - 1 (lanes 0-15) and j0 + rows (lanes 16-31)
        const int top = lane < 16, g = lane & 15;
        if (4 * g < cols)
            group(top ? j0 - 1 : j0 + rows, i0 + 4 * g, top ? 0 : rows + 1, 4 + 4 * g);
    } else if (w == 1) {  // column i0 - 1, rows j0 - 1 .. j0 + min(rows, 31) - 1
        if (lane <= rows)
            single(j0 - 1 + lane, i0 - 1, lane, 3);
    } else if (w == 2) {  // column i0 + cols, rows j0 + 1 .. j0 + rows
        if (lane < rows)
            single(j0 + 1 + lane, i0 + cols, lane + 2, 4 + cols);
    } else if (w == 3) {  // (j0 + 31, i0 - 1) when rows = 32, and (j0, i0 + cols)
        if (lane == 0 && rows == T4Y)
            single(j0 + T4Y - 1, i0 - 1, T4Y, 3);
        else if (lane == 1)
            single(j0, i0 + cols, 1, 4 + cols);
    }
    __syncthreads();
    if (!gon)
        return;
    const long long mo = moff(G, s);
#pragma unroll 1
    for (int r = r0; r < rows && r < r0 + 2; r++) {
        const int j = j0 + r, i = i0 + 4 * gx;
        const int o = (j - 1 + HY) * P + (i - 1 + HX);
        const float *q = sm + (r + 1) * T4W + 4 + 4 * gx;  // (j, i)
        float vxx[4], vyy[4], vxxipjp[4], vyyipjp[4], vyx0[4], vxy0[4], vyxij[4], vxyij[4];
        {
            // (j, i .. i + 4) and (j + 1, i .. i + 4)
            float a[5], b[5];
            lds4(q, a), a[4] = q[4];
            lds4(q + T4W, b), b[4] = q[T4W + 4];
#pragma unroll
            for (int k = 0; k < 4; k++)
                vxx[k] = a[k], vxxipjp[k] = 0.25f * (a[k] + b[k] + a[k + 1] + b[k + 1]);
            lds4(q + T4P, a), a[4] = q[T4P + 4];
            lds4(q + T4P + T4W, b), b[4] = q[T4P + T4W + 4];
#pragma unroll
            for (int k = 0; k < 4; k++)
                vyy[k] = a[k], vyyipjp[k] = 0.25f * (a[k] + b[k] + a[k + 1] + b[k + 1]);
            // (j, i - 1 .. i + 3) and (j - 1, i - 1 .. i + 3)
            lds4(q + 2 * T4P, a + 1), a[0] = q[2 * T4P - 1];
            lds4(q + 2 * T4P - T4W, b + 1), b[0] = q[2 * T4P - T4W - 1];
#pragma unroll
            for (int k = 0; k < 4; k++)
                vyx0[k] = a[k + 1], vyxij[k] = 0.25f * (a[k + 1] + b[k + 1] + a[k] + b[k]);
            lds4(q + 3 * T4P, a + 1), a[0] = q[3 * T4P - 1];
            lds4(q + 3 * T4P - T4W, b + 1), b[0] = q[3 * T4P - T4W - 1];
#pragma unroll
            for (int k = 0; k < 4; k++)
                vxy0[k] = a[k + 1], vxyij[k] = 0.25f * (a[k + 1] + b[k + 1] + a[k] + b[k]);
        }
        tti_update4<VISCO>(G, W, M, s, o, mo, vxx, vyy, vxxipjp, vyyipjp, vyx0, vxy0, vyxij, vxyij);
    }
}

template <int ND, bool VISCO, bool CPML>
__global__ void __launch_bounds__(BX *BY, VISCO ? 2 : 4) k_tti_tiles(Geo G, Wave W, Model M, TtiMap T)
{
    __shared__ __align__(16) float sm[4 * T4P];
    static_assert(sizeof(float) * (CPML ? 2 : 1) * 4 * (BY + 2) * (BX + 2) <= sizeof(sm), "frame tile overflow");
    pdl_begin();
    int b, s;
    block_xs(G, b, s);
    if (b >= T.nframe) {
        b -= T.nframe;
        const int a = b % T.nfx, c = b / T.nfx;
        const int i0 = T.fi0 + a * T4X, j0 = T.fj0 + c * T4Y;
        tti_tile4<ND, VISCO>(G, W, M, s, i0, j0, min(T4X, T.fi1 - i0 + 1), min(T4Y, T.fj1 - j0 + 1), sm);
        return;
    }
    int sx, sy;
    tti_frame_tile(T, b, sx, sy);
    tti_tile<ND, VISCO, CPML>(G, W, M, s, sx * BX + 1, sy * BY + 1, threadIdx.x & (BX - 1), threadIdx.x / BX,
                              reinterpret_cast<float(*)[4][BY + 2][BX + 2]>(sm), T.fi0, T.fi1, T.fj0, T.fj1);
}

// ------------------------------------------------ after the stress update

// psource.c:27-54 / eqsource.c:25-52 restricted to the cells of column i:
// every source of the shot, in order, when the last source's type selects the
// injection (time_loop.c:248-253); a moment tensor also reaches column i-1.
// lt, ka, kb: the shot's last source type and source range (A.last_type[s],
// A.src_off[s], A.src_off[s + 1]), loaded by the caller with its other
// independent loads.
// (si0, sj0): the first source's cell (k = ka), loaded by the caller too; sw:
// its signal around this step (SigWindow), with (sx0, sy0) the stresses at
// its cell as the stress update left them, loaded with the step number.
__device__ __forceinline__ void post_sources(const Geo &G, const Wave &W, const Acq &A, int s, int i, int nt, int lt,
                                             int ka, int kb, int si0, int sj0, const SigWindow &sw, float sx0,
                                             float sy0)
{
    if (lt != 1 && lt != 5)
        return;
    const long long so = (long long)s * G.fsz;
    float *sxx = W.sxx + so, *syy = W.syy + so, *sxy = W.sxy + so;
    const int NT = A.nt;
    for (int k = ka; k < kb; k++) {
        const int si = k == ka ? si0 : A.src_ix[k], sj = k == ka ? sj0 : A.src_iy[k];
        if (si != i && !(lt == 5 && si - 1 == i))
            continue;
        const float *sig = A.signals + (long long)k * NT - 1;  // 1-based: sig[1..NT]
        const long long o = cell(G, sj, si);
        auto sg = [&](int n) { return k == ka ? sw.at(sig, n) : sig[n]; };
        if (lt == 1) {
            // central difference of the signal (psource.c:41-49); a one-step
            // run has no neighbouring sample and injects nothing
            float amp = 0.0f;
            const float d2 = 2.0f * G.dh * G.dh;
            if (NT >= 2) {
                if (nt == 1)
                    amp = sg(2) / d2;
                else if (nt < NT)
                    amp = (sg(nt + 1) - sg(nt - 1)) / d2;
                else
                    amp = -sg(nt - 1) / d2;
            }
            if (k == ka) {  // acoustic: sxx and syy are one array, which takes amp twice
                sxx[o] = sx0 + amp;
                syy[o] = (syy == sxx ? sx0 + amp : sy0) + amp;
            } else {
                sxx[o] += amp;
                syy[o] += amp;
            }
        } else {
            const float amp = A.src_amp[k] * (G.dt / (G.dh * G.dh)) * sg(nt);
            const float m11 = -A.src_sin2[k], m12 = -A.src_cos2[k], m22 = A.src_sin2[k];
            if (si == i) {
                sxx[o] += amp * m11;
                sxy[o] += 0.3f * amp * m12;
                sxy[o - G.pitch] += 0.3f * amp * m12;
                syy[o] += amp * m22;
            } else {
                sxy[o - 1] += 0.3f * amp * m12;
            }
        }
    }
}

// surface_elastic.c:27-90 / surface.c:27-113 at j = 1 for column i.
// Every value is loaded before the first store: the rows written (the
// surface cell's syy, sxx, memory variables, and the mirrored ghost rows
// above it) are none of the rows read below it, and with all loads issued
// together a column costs one memory round trip instead of one per row.
template <int ND, bool VISCO>
__device__ __forceinline__ void post_surface(const Geo &G, const Wave &W, const Model &M, int s, int i)
{
    const int P = G.pitch, j = 1;
    const long long so = (long long)s * G.fsz, mo = moff(G, s);
    const long long o = cell(G, j, i);
    float *sxx = W.sxx + so, *syy = W.syy + so, *sxy = W.sxy + so;
    const float *vx = W.vx + so, *vy = W.vy + so;
    // ---- loads
    float syb[ND], sxb[ND], vxp[ND], vxm[ND], vyp[ND], vym[ND];
#pragma unroll
    for (int m = 1; m <= ND; m++) {
        syb[m - 1] = syy[o + (long long)m * P];
        sxb[m - 1] = sxy[o + (long long)(m - 1) * P];
        vxp[m - 1] = vx[o + m - 1], vxm[m - 1] = vx[o - m];
        vyp[m - 1] = vy[o + (long long)(m - 1) * P], vym[m - 1] = vy[o - (long long)m * P];
    }
    int h = 0;
    long long q = 0;
    float psi = 0.f;
    if (G.abs_type == 1 && !G.boundary) {
        if (i <= G.fw)
            h = i;
        else if (i >= G.nx - G.fw + 1)
            h = i - G.nx + G.fw2;
        if (h) {
            q = ((long long)s * G.ny + (j - 1)) * G.fw2 + (h - 1);
            psi = W.psi_vxx[q];
        }
    }
    const float pu = M.pu[mo + o], ppi = M.ppi[mo + o], sxx0 = sxx[o];
    float taus = 0.f, taup = 0.f, pl[MAXL];
    if (VISCO) {
        taus = M.taus[mo + o], taup = M.taup[mo + o];
#pragma unroll
        for (int l = 0; l < MAXL; l++)
            pl[l] = l < G.L ? W.p[((long long)s * G.L + l) * G.fsz + o] : 0.f;
    }
    // ---- arithmetic and stores, in the reference's order
    syy[o] = 0.0f;
    if (VISCO)
        for (int l = 0; l < G.L; l++)
            W.q[((long long)s * G.L + l) * G.fsz + o] = 0.0f;
    float vxx = 0.f, vyy = 0.f;
#pragma unroll
    for (int m = 1; m <= ND; m++) {
        syy[o - (long long)m * P] = -syb[m - 1];
        sxy[o - (long long)m * P] = -sxb[m - 1];
        vxx += G.hc[m] * (vxp[m - 1] - vxm[m - 1]);
        vyy += G.hc[m] * (vyp[m - 1] - vym[m - 1]);
    }
    vxx *= G.dhi;
    vyy *= G.dhi;
    if (h) {
        float ps = M.b_x[h - 1] * psi + M.a_x[h - 1] * vxx;
        W.psi_vxx[q] = ps;
        vxx = vxx / M.K_x[h - 1] + ps;
    }
    if (!VISCO) {
        float fjm = pu * 2.0f, g = ppi;
        sxx[o] = sxx0 + (-(G.dt * (g - fjm) * (g - fjm) * vxx / g) - (G.dt * (g - fjm) * vyy));
    } else {
        float sump = 0.f;
#pragma unroll
        for (int l = 0; l < MAXL; l++)
            if (l < G.L)
                sump += pl[l];
        float fjm = pu * 2.0f * (1.0f + G.L * taus);
        float g = ppi * (1.0f + G.L * taup);
        float sx = sxx0 + (-(G.dt * (g - fjm) * (g - fjm) * vxx / g) - (G.dt * (g - fjm) * vyy) - (G.dthalbe * sump));
        sump = 0.f;
        float djm = 2.0f * pu * taus, e = ppi * taup;
#pragma unroll
        for (int l = 0; l < MAXL; l++) {
            if (l < G.L) {
                float bjm = M.peta[l] / (1.0f + (M.peta[l] * 0.5f));
                float p = pl[l] + bjm * (((djm - e) * ((fjm / g) - 1.0f) * vxx) - ((djm - e) * vyy));
                W.p[((long long)s * G.L + l) * G.fsz + o] = p;
                sump += p;
            }
        }
        sxx[o] = sx + G.dthalbe * sump;
    }
}

// div / curl of seismo_ssg.c:43-47 for receiver k: the derivatives as the
// stress update left them (CPML-stretched in the frame; psi already holds this
// step's value, so the stretched derivative is d / K + psi). W's CPML memory
// must point at the buffer this step wrote.
template <int ND, bool TTIK>
__device__ __forceinline__ void sample_div_curl(const Geo &G, const Wave &W, const Model &M, const Acq &A, int s,
                                                int k, int ins)
{
    const int i = A.rec_ix[k], j = A.rec_iy[k];
    const long long o = cell(G, j, i);
    const long long so = (long long)s * G.fsz, mo = moff(G, s);
    float vxx, vyx, vxy, vyy;
    {
        op_s<ND>(W.vx + so, W.vy + so, o, G.pitch, G.hc, G.dhi, vxx, vyx, vxy, vyy);
        int xr = xside(G, i), yr = yside(G, j);
        // the EL_TTI right-bottom CPML pass stops at NY-1: raw derivatives there
        if (TTIK && G.el_tti_rb_short && xr == 2 && yr == 2 && j == G.ny)
            xr = yr = 0;
        if (G.abs_type == 1) {
            if (xr) {
                int h = xr == 1 ? i : i - G.nx + G.fw2;
                long long q = ((long long)s * G.ny + (j - 1)) * G.fw2 + (h - 1);
                vxx = vxx / M.K_x[h - 1] + W.psi_vxx[q];
                vyx = vyx / M.K_x_half[h - 1] + W.psi_vyx[q];
            }
            if (yr) {
                int h = yr == 1 ? j : j - G.ny + G.fw2;
                long long q = ((long long)s * G.fw2 + (h - 1)) * G.nx + (i - 1);
                vyy = vyy / M.K_y[h - 1] + W.psi_vyy[q];
                vxy = vxy / M.K_y_half[h - 1] + W.psi_vxy[q];
            }
        }
    }
    float *sec = A.sec + (long long)k * 5 * A.ns + (ins - 1);
    sec[3 * A.ns] = (vxx + vyy) * sqrtf(M.ppi[mo + o]);
    sec[4 * A.ns] = (vxy - vyx) * sqrtf(M.pu[mo + o]);
}

// vx, vy and p of seismo_ssg.c:36-62 for receiver k after the step; (o, vxk,
// vyk): the receiver's cell and its velocities, loaded by the caller (nothing
// after the velocity update writes v).
__device__ __forceinline__ void sample_v_p(const Geo &G, const Wave &W, const Model &M, const Acq &A, int s, int k,
                                           long long o, float vxk, float vyk, int ins, int seismo)
{
    const long long so = (long long)s * G.fsz, mo = moff(G, s);
    float *sec = A.sec + (long long)k * 5 * A.ns + (ins - 1);
    if (seismo == 1 || seismo == 4) {
        sec[0] = vxk;
        sec[A.ns] = vyk;
    }
    if (seismo == 2 || seismo == 4) {
        float p = -W.sxx[so + o] - W.syy[so + o];
        if (seismo == 2)
            sec[2 * A.ns] = p;
        else {
            float ppi = M.ppi[mo + o], pu = M.pu[mo + o];
            sec[2 * A.ns] = ((3.0f * ppi - 4.0f * pu) / (2.0f * ppi - 2.0f * pu)) * p / 3.0f;
        }
    }
}

// The part of a column's post work that depends only on the acquisition,
// which no kernel writes: the shot's last source type and source range, the
// first source's cell, the column's receiver range and its first receiver's
// cell. k_post loads it before it waits for the stress kernel.
struct PostCol {
    int lt, ka, kb, si0, sj0, r0, r1, k0;
    long long o0;
    SigWindow sw;  // the first source's signal around this step, where this column injects it
};

__device__ __forceinline__ PostCol post_acq(const Geo &G, const Acq &A, int i, int s)
{
    PostCol p;
    p.lt = A.last_type[s], p.ka = A.src_off[s], p.kb = A.src_off[s + 1];
    const int *roff = A.rec_col_off ? A.rec_col_off + (long long)s * (G.nx + 1) : nullptr;
    p.r0 = roff ? roff[i - 1] : 0, p.r1 = roff ? roff[i] : 0;
    p.si0 = p.sj0 = p.k0 = 0;
    p.o0 = 0;
    if (p.ka < p.kb) {
        p.si0 = A.src_ix[p.ka], p.sj0 = A.src_iy[p.ka];
        if ((p.lt == 1 || p.lt == 5) && (p.si0 == i || (p.lt == 5 && p.si0 - 1 == i)))
            p.sw.load(G.step_ctr, A.signals + (long long)p.ka * A.nt - 1, A.nt);
    }
    if (p.r0 < p.r1) {
        p.k0 = A.rec_col_idx[p.r0];
        p.o0 = cell(G, A.rec_iy[p.k0], A.rec_ix[p.k0]);
    }
    return p;
}

// Everything of time_loop.c:247-285 after the stress update, one thread per
// column: every operation below reads and writes only cells of its own column
// (a moment tensor's column-(i-1) term is applied by that column's thread), so
// columns are independent. Per column, in the reference's order: div/curl
// sampling (from the stress update's derivatives), source injection, free
// surface, the NaN probe of time_loop.c:44-47, vx/vy/p sampling.
template <int ND, bool VISCO, bool TTIK>
__device__ __forceinline__ void post_column(const Geo &G, Wave W, const Model &M, const Acq &A, int i, int s,
                                            const PostCol &pc)
{
    const int nt = *G.step_ctr;  // the velocity kernel of this step advanced it
    const int seismo = G.seismo;
    psi_buffers(G, W, false);    // TTI: the CPML memory this step's stress update wrote
    // time_loop.c:282: sample at nt = NDT, 2 NDT, ... while nt < NT
    const int ins = (seismo && G.ndt > 0 && nt % G.ndt == 0 && nt < A.nt) ? nt / G.ndt : 0;
    const int r0 = pc.r0, r1 = pc.r1;
    // the column's first receiver's velocities, loaded ahead of the stores below
    const long long so = (long long)s * G.fsz;
    float vx0 = 0.f, vy0 = 0.f, sx0 = 0.f, sy0 = 0.f;
    if (r0 < r1)
        vx0 = W.vx[so + pc.o0], vy0 = W.vy[so + pc.o0];
    if (pc.lt == 1 && pc.ka < pc.kb && pc.si0 == i) {  // the first source's cell, before any injection
        const long long o = so + cell(G, pc.sj0, pc.si0);
        sx0 = W.sxx[o], sy0 = W.syy[o];
    }
    if (ins && (seismo == 3 || seismo == 4))
        for (int r = r0; r < r1; r++)
            sample_div_curl<ND, TTIK>(G, W, M, A, s, A.rec_col_idx[r], ins);
    post_sources(G, W, A, s, i, nt, pc.lt, pc.ka, pc.kb, pc.si0, pc.sj0, pc.sw, sx0, sy0);
    if (G.free_surf)
        post_surface<ND, VISCO>(G, W, M, s, i);
    if (i == (G.nx / 2 > 0 ? G.nx / 2 : 1)) {
        long long pcell = cell(G, G.ny / 2 > 0 ? G.ny / 2 : 1, i);
        if (isnan(W.vy[so + pcell]) && A.status[s] == 0)
            A.status[s] = nt;
    }
    if (ins && seismo != 3)
        for (int r = r0; r < r1; r++) {
            if (r == r0) {
                sample_v_p(G, W, M, A, s, pc.k0, pc.o0, vx0, vy0, ins, seismo);
            } else {
                const int k = A.rec_col_idx[r];
                const long long o = cell(G, A.rec_iy[k], A.rec_ix[k]);
                sample_v_p(G, W, M, A, s, k, o, W.vx[so + o], W.vy[so + o], ins, seismo);
            }
        }
}

template <int ND, bool VISCO, bool TTIK>
__global__ void k_post(Geo G, Wave W, Model M, Acq A)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, s = blockIdx.y;
    PostCol pc{};
    if (i <= G.nx)
        pc = post_acq(G, A, i, s);
    pdl_begin();
    if (i <= G.nx)
        post_column<ND, VISCO, TTIK>(G, W, M, A, i, s, pc);
}

// snap_ssg.c:86-205: one snapshot frame, file order (x outer, y inner).
template <int ND>
__global__ void k_snap(Geo G, Wave W, Model M, float *out, int nsx, int nsy, int idx, int idy, int type,
                       long long frame_stride)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    int s = blockIdx.y;
    if (t >= nsx * nsy)
        return;
    int i = 1 + (t / nsy) * idx, j = 1 + (t % nsy) * idy;
    long long o = cell(G, j, i);
    long long so = (long long)s * G.fsz, mo = moff(G, s);
    const float *vx = W.vx + so, *vy = W.vy + so;
    float *f = out + (long long)s * frame_stride;
    long long n = (long long)nsx * nsy;
    if (type == 1 || type == 4) {
        f[t] = vx[o];
        f[n + t] = vy[o];
    }
    if (type == 2 || type == 4)
        f[2 * n + t] = -W.sxx[so + o] - W.syy[so + o];
    if (type == 3 || type == 4) {
        const int P = G.pitch;
        float vyx = 0.f, vxy = 0.f, vxx = 0.f, vyy = 0.f;
#pragma unroll
        for (int m = 1; m <= ND; m++) {
            vyx += G.hc[m] * (vy[o + m] - vy[o - m + 1]);
            vxy += G.hc[m] * (vx[o + (long long)m * P] - vx[o - (long long)(m - 1) * P]);
            vxx += G.hc[m] * (vx[o + m - 1] - vx[o - m]);
            vyy += G.hc[m] * (vy[o + (long long)(m - 1) * P] - vy[o - (long long)m * P]);
        }
        f[4 * n + t] = (vxy * G.dhi - vyx * G.dhi) * sqrtf(M.pu[mo + o]);
        f[3 * n + t] = (vxx * G.dhi + vyy * G.dhi) * sqrtf(M.ppi[mo + o]);
    }
}

}  // namespace sofi
