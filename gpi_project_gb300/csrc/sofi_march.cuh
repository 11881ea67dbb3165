// sofi_march.cuh -- y-marching velocity and stress kernels (isotropic and VTI).
//
// A block of TX threads owns TX consecutive columns and marches down SY rows.
// Stencils in y read a per-thread register queue of the column (each value
// loaded once per block), stencils in x read one shared-memory row per field
// (TX values plus an ND-wide halo on either side); every per-cell load of a
// row is issued before the arithmetic that uses it. Arithmetic per cell is
// the same as k_update_v / k_update_s (sofi_kernels.cuh), term for term.
#pragma once
#include "sofi_common.cuh"

namespace sofi {

// Load one row of `f` (columns i0-ND .. i0+TX+ND-1) into s[0 .. TX+2ND-1]:
// an active thread's own column comes from `own`; a thread past NX stages its
// column from memory while it is still a ghost column the stencils read
// (NX+1 .. NX+ND: zero, or the periodic copy); halo columns come from memory.
template <int ND, int TX>
__device__ __forceinline__ void stage_row(float *s, const float *__restrict__ rowp, int tx, int i0, int nx, float own,
                                          bool act)
{
    int ic = i0 + tx;
    s[ND + tx] = act ? own : ((ic <= nx + ND) ? __ldg(rowp + ic) : 0.f);
    if (tx < ND) {
        int i = i0 - ND + tx;  // >= 1 - ND: inside the left halo
        s[tx] = __ldg(rowp + i);
    }
    if (tx >= TX - ND) {
        int k = tx - (TX - ND);
        int i = i0 + TX + k;
        s[ND + TX + k] = (i <= nx + ND) ? __ldg(rowp + i) : 0.f;
    }
}

// row pointer such that rowp[i] is cell (j, i) of field f
__device__ __forceinline__ const float *rowptr(const Geo &G, const float *f, int j)
{
    return f + (long long)(j - 1 + HY) * G.pitch + (HX - 1);
}
__device__ __forceinline__ float *rowptr_w(const Geo &G, float *f, int j)
{
    return f + (long long)(j - 1 + HY) * G.pitch + (HX - 1);
}

template <int ND, int TX>
__global__ void __launch_bounds__(TX) k_march_v(Geo G, Wave W, Model M, int SY)
{
    __shared__ float s_xx[TX + 2 * ND], s_xy[TX + 2 * ND];
    const int tx = threadIdx.x;
    const int i0 = blockIdx.x * TX + 1, i = i0 + tx;
    const int j0 = blockIdx.y * SY + 1;
    const int j1 = min(j0 + SY - 1, G.ny);
    const int s = blockIdx.z;
    const bool act = i <= G.nx;
    if (G.step_ctr && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && tx == 0)
        *G.step_ctr += 1;  // as k_update_v
    const long long so = (long long)s * G.fsz, mo = moff(G, s);
    const float *sxx = W.sxx + so, *syy = W.syy + so, *sxy = W.sxy + so;
    float *vx = W.vx + so, *vy = W.vy + so;
    const float *hc = G.hc;
    // queues: qxy[k] = sxy(r - ND + k), k < 2ND; qyy[k] = syy(r - ND + 1 + k)
    float qxy[2 * ND], qyy[2 * ND];
#pragma unroll
    for (int k = 0; k < 2 * ND; k++) {
        qxy[k] = act ? __ldg(rowptr(G, sxy, j0 - ND + k) + i) : 0.f;
        qyy[k] = act ? __ldg(rowptr(G, syy, j0 - ND + 1 + k) + i) : 0.f;
    }
    const int xr = (i <= G.gx2) ? 1 : (i > G.gx3 ? 2 : 0);
    for (int j = j0; j <= j1; j++) {
        // issue this row's loads first
        float nxy = 0.f, nyy = 0.f, cxx = 0.f, ovx = 0.f, ovy = 0.f, rip = 0.f, rjp = 0.f;
        if (act) {
            nxy = __ldg(rowptr(G, sxy, j + ND) + i);
            nyy = __ldg(rowptr(G, syy, j + ND + 1) + i);
            cxx = __ldg(rowptr(G, sxx, j) + i);
            ovx = rowptr(G, vx, j)[i];
            ovy = rowptr(G, vy, j)[i];
            rip = __ldg(rowptr(G, M.prip + mo, j) + i);
            rjp = __ldg(rowptr(G, M.prjp + mo, j) + i);
        }
        __syncthreads();
        stage_row<ND, TX>(s_xx, rowptr(G, sxx, j), tx, i0, G.nx, cxx, act);
        stage_row<ND, TX>(s_xy, rowptr(G, sxy, j), tx, i0, G.nx, qxy[ND], act);
        __syncthreads();
        if (act) {
            const float *a = s_xx + ND + tx, *b = s_xy + ND + tx;
            float sxx_x = hc[1] * (a[1] - a[0]);
            float sxy_x = hc[1] * (b[0] - b[-1]);
            float sxy_y = hc[1] * (qxy[ND] - qxy[ND - 1]);
            float syy_y = hc[1] * (qyy[ND] - qyy[ND - 1]);
#pragma unroll
            for (int m = 2; m <= ND; m++) {
                sxx_x += hc[m] * (a[m] - a[1 - m]);
                sxy_x += hc[m] * (b[m - 1] - b[-m]);
                sxy_y += hc[m] * (qxy[ND + m - 1] - qxy[ND - m]);
                syy_y += hc[m] * (qyy[ND - 1 + m] - qyy[ND - m]);
            }
            int yr = (j <= G.gy2) ? 1 : (j > G.gy3 ? 2 : 0);
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
                float ab = __ldg(rowptr(G, M.absorb + mo, j) + i);
                nvx *= ab;
                nvy *= ab;
            }
            rowptr_w(G, vx, j)[i] = nvx;
            rowptr_w(G, vy, j)[i] = nvy;
        }
#pragma unroll
        for (int k = 0; k < 2 * ND - 1; k++) {
            qxy[k] = qxy[k + 1];
            qyy[k] = qyy[k + 1];
        }
        qxy[2 * ND - 1] = nxy;
        qyy[2 * ND - 1] = nyy;
    }
}

// Stress update of isotropic (elastic / viscoelastic) and VTI media.
// LT > 0: number of relaxation mechanisms fixed at compile time.
template <int ND, int TX, int KIND, bool VISCO, int LT>
__global__ void __launch_bounds__(TX) k_march_s(Geo G, Wave W, Model M, int SY)
{
    __shared__ float s_vx[TX + 2 * ND], s_vy[TX + 2 * ND];
    const int tx = threadIdx.x;
    const int i0 = blockIdx.x * TX + 1, i = i0 + tx;
    const int j0 = blockIdx.y * SY + 1;
    const int j1 = min(j0 + SY - 1, G.ny);
    const int s = blockIdx.z;
    const bool act = i <= G.nx;
    const long long so = (long long)s * G.fsz, mo = moff(G, s);
    const float *vx = W.vx + so, *vy = W.vy + so;
    float *sxx = W.sxx + so, *syy = W.syy + so, *sxy = W.sxy + so;
    const float *hc = G.hc;
    const float dhi = G.dhi;
    // qvx[k] = vx(r - ND + 1 + k), qvy[k] = vy(r - ND + k), k < 2ND
    float qvx[2 * ND], qvy[2 * ND];
#pragma unroll
    for (int k = 0; k < 2 * ND; k++) {
        qvx[k] = act ? __ldg(rowptr(G, vx, j0 - ND + 1 + k) + i) : 0.f;
        qvy[k] = act ? __ldg(rowptr(G, vy, j0 - ND + k) + i) : 0.f;
    }
    const int xr = (i <= G.gx2) ? 1 : (i > G.gx3 ? 2 : 0);
    constexpr int LN = LT > 0 ? LT : 1;
    for (int j = j0; j <= j1; j++) {
        float nvx = 0.f, nvy = 0.f, oxx = 0.f, oyy = 0.f, oxy = 0.f;
        float m0 = 0.f, m1 = 0.f, m2 = 0.f, m3 = 0.f;
        float b0 = 0.f, b1 = 0.f, b2 = 0.f, b3 = 0.f;
        float rr[LN], pp[LN], qq[LN];
        const long long rowo = (long long)(j - 1 + HY) * G.pitch + (HX - 1) + i;
        if (act) {
            nvx = __ldg(rowptr(G, vx, j + ND + 1) + i);
            nvy = __ldg(rowptr(G, vy, j + ND) + i);
            oxx = sxx[rowo], oyy = syy[rowo], oxy = sxy[rowo];
            if (KIND == ISO) {
                m0 = __ldg(M.g + mo + rowo), m1 = __ldg(M.f + mo + rowo), m2 = __ldg(M.fipjp + mo + rowo);
                if (VISCO)
                    b0 = __ldg(M.db + mo + rowo), b1 = __ldg(M.eb + mo + rowo), b2 = __ldg(M.dipb + mo + rowo);
            } else {
                m0 = __ldg(M.c11 + mo + rowo), m1 = __ldg(M.c13 + mo + rowo), m2 = __ldg(M.c33 + mo + rowo);
                m3 = __ldg(M.c55ipjp + mo + rowo);
                if (VISCO) {
                    b0 = __ldg(M.c11b + mo + rowo), b1 = __ldg(M.c13b + mo + rowo), b2 = __ldg(M.c33b + mo + rowo);
                    b3 = __ldg(M.c55ipjpb + mo + rowo);
                }
            }
            if (VISCO && LT > 0) {
#pragma unroll
                for (int l = 0; l < LN; l++) {
                    long long lo = ((long long)s * G.L + l) * G.fsz + rowo;
                    rr[l] = W.r[lo], pp[l] = W.p[lo], qq[l] = W.q[lo];
                }
            }
        }
        __syncthreads();
        stage_row<ND, TX>(s_vx, rowptr(G, vx, j), tx, i0, G.nx, qvx[ND - 1], act);
        stage_row<ND, TX>(s_vy, rowptr(G, vy, j), tx, i0, G.nx, qvy[ND], act);
        __syncthreads();
        if (act) {
            const float *a = s_vx + ND + tx, *b = s_vy + ND + tx;
            float vxx = hc[1] * (a[0] - a[-1]);
            float vyx = hc[1] * (b[1] - b[0]);
            float vxy = hc[1] * (qvx[ND] - qvx[ND - 1]);
            float vyy = hc[1] * (qvy[ND] - qvy[ND - 1]);
#pragma unroll
            for (int m = 2; m <= ND; m++) {
                vxx += hc[m] * (a[m - 1] - a[-m]);
                vyx += hc[m] * (b[m] - b[1 - m]);
                vxy += hc[m] * (qvx[ND - 1 + m] - qvx[ND - m]);
                vyy += hc[m] * (qvy[ND + m - 1] - qvy[ND - m]);
            }
            vxx *= dhi, vyx *= dhi, vxy *= dhi, vyy *= dhi;
            int yr = (j <= G.gy2) ? 1 : (j > G.gy3 ? 2 : 0);
            if (G.abs_type == 1)
                cpml_s(G, W, M, s, i, j, xr, yr, vxx, vyx, vxy, vyy, true);
            float u1, u2, u3;
            if (KIND == ISO) {
                u1 = m2 * (vyx + vxy);
                float gd = m0 * (vxx + vyy);
                u2 = gd - 2.0f * m1 * vyy;
                u3 = gd - 2.0f * m1 * vxx;
            } else {
                u1 = m3 * (vxy + vyx);
                u2 = m0 * vxx + m1 * vyy;
                u3 = m1 * vxx + m2 * vyy;
            }
            if (VISCO) {
                float sro = 0.f, spo = 0.f, sqo = 0.f, sr = 0.f, sp = 0.f, sq = 0.f;
                const int L = LT > 0 ? LT : G.L;
#pragma unroll
                for (int l = 0; l < (LT > 0 ? LT : MAXL); l++) {
                    if (LT == 0 && l >= L)
                        break;
                    long long lo = ((long long)s * G.L + l) * G.fsz + rowo;
                    float r = LT > 0 ? rr[l] : W.r[lo], p = LT > 0 ? pp[l] : W.p[lo], q = LT > 0 ? qq[l] : W.q[lo];
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
                    W.r[lo] = r, W.p[lo] = p, W.q[lo] = q;
                    sr += r, sp += p, sq += q;
                }
                u1 += G.dthalbe * (sro + sr);
                u2 += G.dthalbe * (spo + sp);
                u3 += G.dthalbe * (sqo + sq);
            }
            float nxy = oxy + u1, nxx = oxx + u2, nyy = oyy + u3;
            if (G.abs_type == 2 && (xr | yr)) {
                float ab = __ldg(M.absorb + mo + rowo);
                nxy *= ab, nyy *= ab, nxx *= ab;
            }
            sxy[rowo] = nxy;
            sxx[rowo] = nxx;
            syy[rowo] = nyy;
        }
#pragma unroll
        for (int k = 0; k < 2 * ND - 1; k++) {
            qvx[k] = qvx[k + 1];
            qvy[k] = qvy[k + 1];
        }
        qvx[2 * ND - 1] = nvx;
        qvy[2 * ND - 1] = nvy;
    }
}

}  // namespace sofi
