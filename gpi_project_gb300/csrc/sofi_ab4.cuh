// sofi_ab4.cuh -- 4th-order Adams-Bashforth time stepping (FDORDER_TIME = 4) of
// the reference's elastic and viscoelastic isotropic updates:
//   update_v_interior_4.c / update_v_PML_4.c / update_v_abs_4.c with
//   wavefield_update_v_4.c, update_s_{elastic,visc}_{interior,PML,abs}_4.c with
//   wavefield_update_s_{el,visc}_4.c, and the history shifts of time_loop.c:89-91,
//   228-244 (shift_var2 / shift_var3, util.c:89-109).
//
// The reference rotates four history arrays by pointer after each step. Here
// every history holds four buffers and the level is picked on the device from
// the step number n (the counter that k_ab4_begin advances): level 1 of a
// derivative history is buffer n mod 4, level k buffer (n - k + 1) mod 4; the
// memory variables' current level is buffer (n - 1) mod 4 and the new values
// go to buffer n mod 4. Launch arguments are the same every step, so the step
// graph replays as for the second-order loop.
//
// The reference's 4th-order velocity CPML driver (update_v_PML_4.c) runs the
// CPML recursion in the left frame and in all four corners but never updates
// the velocity there; k_update_v_ab4 does the same. The reference evaluates a
// few terms in double (2.0 * f * sumyy * dhi, DT / 2.0); here they are float.
#pragma once
#include "sofi_kernels.cuh"

namespace sofi {

// Adams-Bashforth coefficients, float as the reference declares them
constexpr float kAB1 = (float)(13.0 / 12.0), kAB2 = (float)(-5.0 / 24.0), kAB3 = (float)(1.0 / 6.0),
                kAB4 = (float)(-1.0 / 24.0);

// One thread: the step about to be computed gets its number (force sources
// already read counter + 1 before this launch).
static __global__ void k_ab4_begin(Geo G)
{
    *G.step_ctr += 1;
}

template <int ND>
__global__ void __launch_bounds__(BX *BY) k_update_v_ab4(Geo G, Wave W, Model M)
{
    int bx, s;
    block_xs(G, bx, s);
    const int i = bx * BX + threadIdx.x + 1;
    const int j = blockIdx.y * BY + threadIdx.y + 1;
    if (i > G.nx || j > G.ny)
        return;
    const int n = *G.step_ctr;
    const long long so = (long long)s * G.fsz, mo = moff(G, s);
    const long long o = cell(G, j, i);
    float sxx_x, sxy_x, sxy_y, syy_y;
    op_v<ND>(W.sxx + so, W.syy + so, W.sxy + so, o, G.pitch, G.hc, sxx_x, sxy_x, sxy_y, syy_y);
    const int xr = xside(G, i), yr = yside(G, j);
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
        if (xr == 1 || (xr && yr))
            return;  // update_v_PML_4.c: no update in the left frame and the corners
    }
    const long long L1 = (n & 3) * W.ab_lvl, L2 = ((n - 1) & 3) * W.ab_lvl, L3 = ((n - 2) & 3) * W.ab_lvl,
                    L4 = ((n - 3) & 3) * W.ab_lvl;
    const long long so4 = so + o;
    const float s1x = sxx_x + sxy_y, s1y = sxy_x + syy_y;
    W.svx4[L1 + so4] = s1x;
    W.svy4[L1 + so4] = s1y;
    float nvx = W.vx[so4] + (kAB1 * s1x + kAB2 * W.svx4[L2 + so4] + kAB3 * W.svx4[L3 + so4] +
                             kAB4 * W.svx4[L4 + so4]) * G.dtdh * M.prip[mo + o];
    float nvy = W.vy[so4] + (kAB1 * s1y + kAB2 * W.svy4[L2 + so4] + kAB3 * W.svy4[L3 + so4] +
                             kAB4 * W.svy4[L4 + so4]) * G.dtdh * M.prjp[mo + o];
    if (G.abs_type == 2 && (xr | yr)) {
        const float a = M.absorb[mo + o];
        nvx *= a, nvy *= a;
    }
    W.vx[so4] = nvx;
    W.vy[so4] = nvy;
}

template <int ND, bool VISCO>
__global__ void __launch_bounds__(BX *BY) k_update_s_ab4(Geo G, Wave W, Model M)
{
    int bx, s;
    block_xs(G, bx, s);
    const int i = bx * BX + threadIdx.x + 1;
    const int j = blockIdx.y * BY + threadIdx.y + 1;
    if (i > G.nx || j > G.ny)
        return;
    const int n = *G.step_ctr;
    const long long so = (long long)s * G.fsz, mo = moff(G, s);
    const long long o = cell(G, j, i), so4 = so + o;
    float vxx, vyx, vxy, vyy;
    op_s<ND>(W.vx + so, W.vy + so, o, G.pitch, G.hc, G.dhi, vxx, vyx, vxy, vyy);
    const int xr = xside(G, i), yr = yside(G, j);
    if (G.abs_type == 1)
        cpml_s(G, W, M, s, i, j, xr, yr, vxx, vyx, vxy, vyy, true);
    const long long L1 = (n & 3) * W.ab_lvl, L2 = ((n - 1) & 3) * W.ab_lvl, L3 = ((n - 2) & 3) * W.ab_lvl,
                    L4 = ((n - 3) & 3) * W.ab_lvl;
    // the stored derivatives times DH (wavefield_update_s_el_4.c:40-43)
    const float h1xx = vxx * G.dh, h1yy = vyy * G.dh, h1xy = vxy * G.dh, h1yx = vyx * G.dh;
    W.hxx4[L1 + so4] = h1xx, W.hyy4[L1 + so4] = h1yy, W.hxy4[L1 + so4] = h1xy, W.hyx4[L1 + so4] = h1yx;
    const float sumxx = kAB1 * h1xx + kAB2 * W.hxx4[L2 + so4] + kAB3 * W.hxx4[L3 + so4] + kAB4 * W.hxx4[L4 + so4];
    const float sumyy = kAB1 * h1yy + kAB2 * W.hyy4[L2 + so4] + kAB3 * W.hyy4[L3 + so4] + kAB4 * W.hyy4[L4 + so4];
    const float sumxy = kAB1 * h1xy + kAB2 * W.hxy4[L2 + so4] + kAB3 * W.hxy4[L3 + so4] + kAB4 * W.hxy4[L4 + so4];
    const float sumyx = kAB1 * h1yx + kAB2 * W.hyx4[L2 + so4] + kAB3 * W.hyx4[L3 + so4] + kAB4 * W.hyx4[L4 + so4];
    const float dhi = G.dhi4;  // 1.0 / DH rounded to float (wavefield_update_s_*_4.c)
    const float g = M.g[mo + o], f = M.f[mo + o], fipjp = M.fipjp[mo + o];
    float u1, u2, u3;
    if (!VISCO) {
        u1 = fipjp * (sumxy + sumyx) * dhi;
        u2 = ((g * (sumxx + sumyy)) - (2.0f * f * sumyy)) * dhi;
        u3 = ((g * (sumxx + sumyy)) - (2.0f * f * sumxx)) * dhi;
    } else {
        // wavefield_update_s_visc_4.c:48-83; memory variables of level 4 are
        // replaced by the new values
        const float db = M.db[mo + o], eb = M.eb[mo + o], dipb = M.dipb[mo + o];
        const long long C1 = ((n - 1) & 3) * W.ab_mlvl, C2 = ((n - 2) & 3) * W.ab_mlvl,
                        C3 = ((n - 3) & 3) * W.ab_mlvl, C4 = (n & 3) * W.ab_mlvl;
        float sro = 0.f, spo = 0.f, sqo = 0.f, sr = 0.f, sp = 0.f, sq = 0.f;
        for (int l = 0; l < G.L; l++) {
            const long long lo = ((long long)s * G.L + l) * G.fsz + o;
            const float r = W.r[C1 + lo], r2 = W.r[C2 + lo], r3 = W.r[C3 + lo], r4 = W.r[C4 + lo];
            const float p = W.p[C1 + lo], p2 = W.p[C2 + lo], p3 = W.p[C3 + lo], p4 = W.p[C4 + lo];
            const float q = W.q[C1 + lo], q2 = W.q[C2 + lo], q3 = W.q[C3 + lo], q4 = W.q[C4 + lo];
            sro += kAB1 * r + kAB2 * r2 + kAB3 * r3 + kAB4 * r4;
            spo += kAB1 * p + kAB2 * p2 + kAB3 * p3 + kAB4 * p4;
            sqo += kAB1 * q + kAB2 * q2 + kAB3 * q3 + kAB4 * q4;
            const float pe = M.peta[l], bb = M.bip[l], cc = M.cip[l];
            const float ct = 2.0f * (1.0f - cc) / kAB1;
            const float dip = dipb * pe, d = db * pe, e = eb * pe;
            const float nr = bb * (r * cc - ct * kAB2 * (r + r2) - ct * kAB3 * (r2 + r3) - ct * kAB4 * (r3 + r4) -
                                   (dip * (sumxy + sumyx) * dhi));
            const float np = bb * (p * cc - ct * kAB2 * (p + p2) - ct * kAB3 * (p2 + p3) - ct * kAB4 * (p3 + p4) -
                                   (e * (sumxx + sumyy) * dhi) + (2.0f * d * sumyy * dhi));
            const float nq = bb * (q * cc - ct * kAB2 * (q + q2) - ct * kAB3 * (q2 + q3) - ct * kAB4 * (q3 + q4) -
                                   (e * (sumxx + sumyy) * dhi) + (2.0f * d * sumxx * dhi));
            W.r[C4 + lo] = nr, W.p[C4 + lo] = np, W.q[C4 + lo] = nq;
            sr += kAB1 * nr + kAB2 * r + kAB3 * r2 + kAB4 * r3;
            sp += kAB1 * np + kAB2 * p + kAB3 * p2 + kAB4 * p3;
            sq += kAB1 * nq + kAB2 * q + kAB3 * q2 + kAB4 * q3;
        }
        const float dthalbe = G.dthalbe;
        u1 = (fipjp * (sumxy + sumyx)) * dhi + (dthalbe * (sro + sr));
        u2 = (g * (sumxx + sumyy) * dhi) - (2.0f * f * sumyy * dhi) + (dthalbe * (spo + sp));
        u3 = (g * (sumxx + sumyy) * dhi) - (2.0f * f * sumxx * dhi) + (dthalbe * (sqo + sq));
    }
    float nxy = W.sxy[so4] + u1, nxx = W.sxx[so4] + u2, nyy = W.syy[so4] + u3;
    if (G.abs_type == 2 && (xr | yr)) {
        const float a = M.absorb[mo + o];
        nxy *= a, nyy *= a, nxx *= a;
    }
    W.sxy[so4] = nxy;
    W.sxx[so4] = nxx;
    W.syy[so4] = nyy;
}

// ---- four cells per thread in x: every field, history level and memory
// variable moves as 16-byte vectors, the derivatives come from the vector
// stencils of the second-order kernels (v_derivs / s_derivs, the same
// expressions as op_v / op_s); per cell the arithmetic above, term by term.

template <int ND>
__global__ void __launch_bounds__(BX *BY, 3) k_update_v_ab4w(Geo G, Wave W, Model M)
{
    constexpr int VW = 4;
    int bx, s;
    block_xs(G, bx, s);
    const int i = (bx * BX + threadIdx.x) * VW + 1;
    const int j = blockIdx.y * BY + threadIdx.y + 1;
    if (i > G.nx || j > G.ny)
        return;
    const int n = *G.step_ctr;
    const int P = G.pitch;
    const int o = (j - 1 + HY) * P + (i - 1 + HX);  // VW-aligned
    const long long so = (long long)s * G.fsz, mo = moff(G, s), so4 = so + o;
    const float *__restrict__ sxx = W.sxx + so;
    const float *__restrict__ sxy = W.sxy + so;
    const float *__restrict__ syy = W.syy + so;
    float sxx_x[VW], sxy_x[VW], sxy_y[VW], syy_y[VW];
    v_derivs<ND, VW, true>(
        G,
        [&](int f, int dy, int dx, float *out) {
            ldv<VW>((f == 0 ? sxx : f == 1 ? sxy : syy) + o + dy * P + dx, out);
        },
        sxx_x, sxy_x, sxy_y, syy_y);
    const long long L1 = (n & 3) * W.ab_lvl, L2 = ((n - 1) & 3) * W.ab_lvl, L3 = ((n - 2) & 3) * W.ab_lvl,
                    L4 = ((n - 3) & 3) * W.ab_lvl;
    float ox[VW], oy[VW], rp[VW], rq[VW], x2[VW], x3[VW], x4[VW], y2[VW], y3[VW], y4[VW];
    ldv_rw<VW>(W.vx + so4, ox), ldv_rw<VW>(W.vy + so4, oy);
    ldv<VW>(M.prip + mo + o, rp), ldv<VW>(M.prjp + mo + o, rq);
    ldv<VW>(W.svx4 + L2 + so4, x2), ldv<VW>(W.svx4 + L3 + so4, x3), ldv<VW>(W.svx4 + L4 + so4, x4);
    ldv<VW>(W.svy4 + L2 + so4, y2), ldv<VW>(W.svy4 + L3 + so4, y3), ldv<VW>(W.svy4 + L4 + so4, y4);
    const int yr = yside(G, j);
    float s1x[VW], s1y[VW], nvx[VW], nvy[VW];
    bool upd[VW];
    int nupd = 0;
#pragma unroll
    for (int c = 0; c < VW; c++) {
        const int ic = i + c;
        upd[c] = ic <= G.nx;
        const int xr = upd[c] ? xside(G, ic) : 0;
        float fx = sxx_x[c], fxy = sxy_x[c], fyx = sxy_y[c], fy = syy_y[c];
        if (G.abs_type == 1 && upd[c]) {
            if (xr) {
                int h = xr == 1 ? ic : ic - G.nx + G.fw2;
                long long q = ((long long)s * G.ny + (j - 1)) * G.fw2 + (h - 1);
                float ps = M.b_x_half[h - 1] * W.psi_sxx_x[q] + M.a_x_half[h - 1] * fx;
                W.psi_sxx_x[q] = ps;
                fx = fx / M.K_x_half[h - 1] + ps;
                float py = M.b_x[h - 1] * W.psi_sxy_x[q] + M.a_x[h - 1] * fxy;
                W.psi_sxy_x[q] = py;
                fxy = fxy / M.K_x[h - 1] + py;
            }
            if (yr) {
                int h = yr == 1 ? j : j - G.ny + G.fw2;
                long long q = ((long long)s * G.fw2 + (h - 1)) * G.nx + (ic - 1);
                float ps = M.b_y_half[h - 1] * W.psi_syy_y[q] + M.a_y_half[h - 1] * fy;
                W.psi_syy_y[q] = ps;
                fy = fy / M.K_y_half[h - 1] + ps;
                float py = M.b_y[h - 1] * W.psi_sxy_y[q] + M.a_y[h - 1] * fyx;
                W.psi_sxy_y[q] = py;
                fyx = fyx / M.K_y[h - 1] + py;
            }
            if (xr == 1 || (xr && yr))
                upd[c] = false;  // update_v_PML_4.c: no update in the left frame and the corners
        }
        s1x[c] = fx + fyx, s1y[c] = fxy + fy;
        nvx[c] = ox[c] + (kAB1 * s1x[c] + kAB2 * x2[c] + kAB3 * x3[c] + kAB4 * x4[c]) * G.dtdh * rp[c];
        nvy[c] = oy[c] + (kAB1 * s1y[c] + kAB2 * y2[c] + kAB3 * y3[c] + kAB4 * y4[c]) * G.dtdh * rq[c];
        if (G.abs_type == 2 && (xr | yr)) {
            const float a = __ldg(M.absorb + mo + o + c);
            nvx[c] *= a, nvy[c] *= a;
        }
        nupd += upd[c];
    }
    if (nupd == VW) {
        stv<VW>(W.svx4 + L1 + so4, s1x), stv<VW>(W.svy4 + L1 + so4, s1y);
        stv<VW>(W.vx + so4, nvx), stv<VW>(W.vy + so4, nvy);
    } else {
#pragma unroll
        for (int c = 0; c < VW; c++)
            if (upd[c]) {
                W.svx4[L1 + so4 + c] = s1x[c], W.svy4[L1 + so4 + c] = s1y[c];
                W.vx[so4 + c] = nvx[c], W.vy[so4 + c] = nvy[c];
            }
    }
}

template <int ND, bool VISCO>
__global__ void __launch_bounds__(BX *BY, VISCO ? 2 : 3) k_update_s_ab4w(Geo G, Wave W, Model M)
{
    constexpr int VW = 4;
    int bx, s;
    block_xs(G, bx, s);
    const int i = (bx * BX + threadIdx.x) * VW + 1;
    const int j = blockIdx.y * BY + threadIdx.y + 1;
    if (i > G.nx || j > G.ny)
        return;
    const int n = *G.step_ctr;
    const int P = G.pitch;
    const int o = (j - 1 + HY) * P + (i - 1 + HX);  // VW-aligned
    const long long so = (long long)s * G.fsz, mo = moff(G, s), so4 = so + o;
    const float *__restrict__ vx = W.vx + so;
    const float *__restrict__ vy = W.vy + so;
    float vxx[VW], vyx[VW], vxy[VW], vyy[VW];
    s_derivs<ND, VW>(
        G, [&](int f, int dy, int dx, float *out) { ldv<VW>((f == 0 ? vx : vy) + o + dy * P + dx, out); }, vxx, vyx,
        vxy, vyy);
    const int yr = yside(G, j);
    int xr[VW];
#pragma unroll
    for (int c = 0; c < VW; c++) {
        xr[c] = i + c <= G.nx ? xside(G, i + c) : 0;
        if (G.abs_type == 1 && i + c <= G.nx)
            cpml_s(G, W, M, s, i + c, j, xr[c], yr, vxx[c], vyx[c], vxy[c], vyy[c], true);
    }
    const long long L1 = (n & 3) * W.ab_lvl, L2 = ((n - 1) & 3) * W.ab_lvl, L3 = ((n - 2) & 3) * W.ab_lvl,
                    L4 = ((n - 3) & 3) * W.ab_lvl;
    // the stored derivatives times DH (wavefield_update_s_el_4.c:40-43)
    float h1xx[VW], h1yy[VW], h1xy[VW], h1yx[VW], sumxx[VW], sumyy[VW], sumxy[VW], sumyx[VW];
    {
        float a2[VW], a3[VW], a4[VW];
#pragma unroll
        for (int c = 0; c < VW; c++)
            h1xx[c] = vxx[c] * G.dh, h1yy[c] = vyy[c] * G.dh, h1xy[c] = vxy[c] * G.dh, h1yx[c] = vyx[c] * G.dh;
#define SOFI_AB4_SUM(H, H1, SUM)                                                                                 \
    ldv<VW>(W.H + L2 + so4, a2), ldv<VW>(W.H + L3 + so4, a3), ldv<VW>(W.H + L4 + so4, a4);                    \
    _Pragma("unroll") for (int c = 0; c < VW; c++) SUM[c] = kAB1 * H1[c] + kAB2 * a2[c] + kAB3 * a3[c] + kAB4 * a4[c];
        SOFI_AB4_SUM(hxx4, h1xx, sumxx)
        SOFI_AB4_SUM(hyy4, h1yy, sumyy)
        SOFI_AB4_SUM(hxy4, h1xy, sumxy)
        SOFI_AB4_SUM(hyx4, h1yx, sumyx)
#undef SOFI_AB4_SUM
    }
    const bool whole = i + VW - 1 <= G.nx;
    if (whole) {
        stv<VW>(W.hxx4 + L1 + so4, h1xx), stv<VW>(W.hyy4 + L1 + so4, h1yy);
        stv<VW>(W.hxy4 + L1 + so4, h1xy), stv<VW>(W.hyx4 + L1 + so4, h1yx);
    } else {
#pragma unroll
        for (int c = 0; c < VW; c++)
            if (i + c <= G.nx) {
                W.hxx4[L1 + so4 + c] = h1xx[c], W.hyy4[L1 + so4 + c] = h1yy[c];
                W.hxy4[L1 + so4 + c] = h1xy[c], W.hyx4[L1 + so4 + c] = h1yx[c];
            }
    }
    const float dhi = G.dhi4;  // 1.0 / DH rounded to float (wavefield_update_s_*_4.c)
    float g[VW], f[VW], fipjp[VW], u1[VW], u2[VW], u3[VW];
    if (!VISCO) {
        ldv<VW>(M.g + mo + o, g), ldv<VW>(M.f + mo + o, f), ldv<VW>(M.fipjp + mo + o, fipjp);
#pragma unroll
        for (int c = 0; c < VW; c++) {
            u1[c] = fipjp[c] * (sumxy[c] + sumyx[c]) * dhi;
            u2[c] = ((g[c] * (sumxx[c] + sumyy[c])) - (2.0f * f[c] * sumyy[c])) * dhi;
            u3[c] = ((g[c] * (sumxx[c] + sumyy[c])) - (2.0f * f[c] * sumxx[c])) * dhi;
        }
    } else {
        // wavefield_update_s_visc_4.c:48-83; memory variables of level 4 are
        // replaced by the new values
        float db[VW], eb[VW], dipb[VW];
        ldv<VW>(M.db + mo + o, db), ldv<VW>(M.eb + mo + o, eb), ldv<VW>(M.dipb + mo + o, dipb);
        const long long C1 = ((n - 1) & 3) * W.ab_mlvl, C2 = ((n - 2) & 3) * W.ab_mlvl,
                        C3 = ((n - 3) & 3) * W.ab_mlvl, C4 = (n & 3) * W.ab_mlvl;
        float sro[VW], spo[VW], sqo[VW], sr[VW], sp[VW], sq[VW];
#pragma unroll
        for (int c = 0; c < VW; c++)
            sro[c] = spo[c] = sqo[c] = sr[c] = sp[c] = sq[c] = 0.f;
        for (int l = 0; l < G.L; l++) {
            const long long lo = ((long long)s * G.L + l) * G.fsz + o;
            float r[VW], r2[VW], r3[VW], r4[VW], p[VW], p2[VW], p3[VW], p4[VW], q[VW], q2[VW], q3[VW], q4[VW];
            ldv<VW>(W.r + C1 + lo, r), ldv<VW>(W.r + C2 + lo, r2), ldv<VW>(W.r + C3 + lo, r3);
            ldv_rw<VW>(W.r + C4 + lo, r4);
            ldv<VW>(W.p + C1 + lo, p), ldv<VW>(W.p + C2 + lo, p2), ldv<VW>(W.p + C3 + lo, p3);
            ldv_rw<VW>(W.p + C4 + lo, p4);
            ldv<VW>(W.q + C1 + lo, q), ldv<VW>(W.q + C2 + lo, q2), ldv<VW>(W.q + C3 + lo, q3);
            ldv_rw<VW>(W.q + C4 + lo, q4);
            const float pe = M.peta[l], bb = M.bip[l], cc = M.cip[l];
            const float ct = 2.0f * (1.0f - cc) / kAB1;
            float nr[VW], np[VW], nq[VW];
#pragma unroll
            for (int c = 0; c < VW; c++) {
                sro[c] += kAB1 * r[c] + kAB2 * r2[c] + kAB3 * r3[c] + kAB4 * r4[c];
                spo[c] += kAB1 * p[c] + kAB2 * p2[c] + kAB3 * p3[c] + kAB4 * p4[c];
                sqo[c] += kAB1 * q[c] + kAB2 * q2[c] + kAB3 * q3[c] + kAB4 * q4[c];
                const float dip = dipb[c] * pe, d = db[c] * pe, e = eb[c] * pe;
                nr[c] = bb * (r[c] * cc - ct * kAB2 * (r[c] + r2[c]) - ct * kAB3 * (r2[c] + r3[c]) -
                              ct * kAB4 * (r3[c] + r4[c]) - (dip * (sumxy[c] + sumyx[c]) * dhi));
                np[c] = bb * (p[c] * cc - ct * kAB2 * (p[c] + p2[c]) - ct * kAB3 * (p2[c] + p3[c]) -
                              ct * kAB4 * (p3[c] + p4[c]) - (e * (sumxx[c] + sumyy[c]) * dhi) +
                              (2.0f * d * sumyy[c] * dhi));
                nq[c] = bb * (q[c] * cc - ct * kAB2 * (q[c] + q2[c]) - ct * kAB3 * (q2[c] + q3[c]) -
                              ct * kAB4 * (q3[c] + q4[c]) - (e * (sumxx[c] + sumyy[c]) * dhi) +
                              (2.0f * d * sumxx[c] * dhi));
                sr[c] += kAB1 * nr[c] + kAB2 * r[c] + kAB3 * r2[c] + kAB4 * r3[c];
                sp[c] += kAB1 * np[c] + kAB2 * p[c] + kAB3 * p2[c] + kAB4 * p3[c];
                sq[c] += kAB1 * nq[c] + kAB2 * q[c] + kAB3 * q2[c] + kAB4 * q3[c];
            }
            if (whole) {
                stv<VW>(W.r + C4 + lo, nr), stv<VW>(W.p + C4 + lo, np), stv<VW>(W.q + C4 + lo, nq);
            } else {
#pragma unroll
                for (int c = 0; c < VW; c++)
                    if (i + c <= G.nx)
                        W.r[C4 + lo + c] = nr[c], W.p[C4 + lo + c] = np[c], W.q[C4 + lo + c] = nq[c];
            }
        }
        const float dthalbe = G.dthalbe;
        ldv<VW>(M.g + mo + o, g), ldv<VW>(M.f + mo + o, f), ldv<VW>(M.fipjp + mo + o, fipjp);
#pragma unroll
        for (int c = 0; c < VW; c++) {
            u1[c] = (fipjp[c] * (sumxy[c] + sumyx[c])) * dhi + (dthalbe * (sro[c] + sr[c]));
            u2[c] = (g[c] * (sumxx[c] + sumyy[c]) * dhi) - (2.0f * f[c] * sumyy[c] * dhi) + (dthalbe * (spo[c] + sp[c]));
            u3[c] = (g[c] * (sumxx[c] + sumyy[c]) * dhi) - (2.0f * f[c] * sumxx[c] * dhi) + (dthalbe * (sqo[c] + sq[c]));
        }
    }
    float oxy[VW], oxx[VW], oyy[VW];
    ldv_rw<VW>(W.sxy + so4, oxy), ldv_rw<VW>(W.sxx + so4, oxx), ldv_rw<VW>(W.syy + so4, oyy);
#pragma unroll
    for (int c = 0; c < VW; c++) {
        oxy[c] = oxy[c] + u1[c], oxx[c] = oxx[c] + u2[c], oyy[c] = oyy[c] + u3[c];
        if (G.abs_type == 2 && (xr[c] | yr)) {
            const float a = __ldg(M.absorb + mo + o + c);
            oxy[c] *= a, oyy[c] *= a, oxx[c] *= a;
        }
    }
    if (whole) {
        stv<VW>(W.sxy + so4, oxy), stv<VW>(W.sxx + so4, oxx), stv<VW>(W.syy + so4, oyy);
    } else {
#pragma unroll
        for (int c = 0; c < VW; c++)
            if (i + c <= G.nx)
                W.sxy[so4 + c] = oxy[c], W.sxx[so4 + c] = oxx[c], W.syy[so4 + c] = oyy[c];
    }
}

}  // namespace sofi
