// sofi_common.cuh -- types, layout and inline device helpers shared by the kernels.
//
// One time step of the reference's time_loop (src/time_loop.c:42-322) is
//   k_force_src    force sources before the velocity update (update_v_interior.c:49-71)
//   k_update_vw    velocity update, 2 or 4 cells per thread (k_update_v: one cell, or
//                  R rows per thread), CPML / damping frame by predicate
//                  (update_v_interior.c, update_v_PML.c, update_v_abs.c); advances
//                  the device step counter
//   k_wrap_x       periodic x only: ghost columns (exchange_v.c / exchange_s.c, one rank)
//   k_update_sw    ISO / VTI stress update, 2 or 4 cells per thread (k_update_s: one
//                  cell), velocity derivatives recomputed from v in registers
//                  (v_derivatives.c fused away), CPML / damping by predicate
//   k_tti_fused    TTI stress update in one pass: derivatives of the tile and its
//                  ring in shared memory, the reference's region order for the
//                  4-point averages (update_s_elastic_TTI_PML.c); k_tti_deriv +
//                  k_update_s_tti are the two-kernel form
//   k_post         per column: div/curl sampling, explosive / moment-tensor sources,
//                  free surface, NaN probe, v/p sampling (psource.c, eqsource.c,
//                  surface_elastic.c, surface.c, seismo_ssg.c)
//   k_snap         snapshot frame (snap_ssg.c)
// The kernels live in sofi_kernels.cuh; sofi_velocity.cu, sofi_stress_*.cu and
// sofi_tti.cu instantiate them in separate translation units.
//
// Layout: every 2-D field is a padded [NY + 2*HY][pitch] float array with the
// interior cell (j, i) at ((j-1+HY) * pitch + (i-1+HX)); HX = HY = 8 >= ND + 1,
// pitch a multiple of 32 floats. The shot index is the slowest dimension
// (field = base + shot * fsz). Ghost cells stay zero (or hold the periodic
// copy), as the reference's edge ranks.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>

namespace sofi {

// Programmatic dependent launch. The step's main kernels are launched with
// programmatic stream serialisation (launch_pdl), so the GPU may schedule one
// while the previous kernel of the stream is still running. Each such kernel
// calls pdl_begin() before touching the wave fields: griddepcontrol.wait returns once
// the previous kernel has completed and its writes are visible (a no-op after
// an ordinary launch), then launch_dependents lets the next kernel be
// scheduled. The launch of one kernel thus overlaps the tail of the last, and
// no kernel reads or writes a wave field before its predecessor has finished
// (k_post and k_force_src load acquisition and model arrays, which no kernel
// writes, before their wait).
__device__ __forceinline__ void pdl_begin()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// A source's signal samples c0 - 1 .. c0 + 2 (1-based, 0 outside 1 .. NT),
// loaded before griddepcontrol.wait, where c0 is the step counter read there:
// the velocity kernel of the step may be advancing it, so c0 is this step or
// the one before, and the samples a step's injection needs are then in the
// window. at() takes a sample from the window where its index lies in it and
// loads it otherwise, so the result does not depend on the value read.
struct SigWindow {
    int c0;
    float w[4];
    __device__ __forceinline__ void load(const int *step_ctr, const float *sig, int NT)
    {
        asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(c0) : "l"(step_ctr));
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int n = c0 - 1 + q;
            w[q] = (n >= 1 && n <= NT) ? sig[n] : 0.f;
        }
    }
    __device__ __forceinline__ float at(const float *sig, int n) const
    {
        const int q = n - c0 + 1;  // selected, not indexed: w stays in registers
        if (q < 0 || q > 3)
            return sig[n];
        return q == 0 ? w[0] : (q == 1 ? w[1] : (q == 2 ? w[2] : w[3]));
    }
};

// Whether launch_pdl uses programmatic serialisation on this host thread; the
// context whose step is being launched sets it (off: ordinary launches of the
// same kernels).
inline bool &pdl_flag()
{
    static thread_local bool on = true;
    return on;
}

// Launch k on st with programmatic stream serialisation (k begins with
// pdl_begin()).
template <typename... KArgs, typename... Args>
inline void launch_pdl(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args... args)
{
    if (!pdl_flag()) {
        k<<<grid, block, smem, st>>>(args...);
        return;
    }
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid, cfg.blockDim = block, cfg.dynamicSmemBytes = smem, cfg.stream = st;
    cfg.attrs = at, cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k, args...);  // an error stays with cudaGetLastError()
}

constexpr int HX = 8;
constexpr int HY = 8;
constexpr int MAXL = 8;
constexpr int BX = 32;  // threads per block in x
constexpr int BY = 8;   // threads per block in y

enum Kind { ISO = 0, VTI = 1, TTI = 2, AC = 3 };  // AC: acoustic, one pressure field

struct Geo {
    int nx, ny, pitch, nshots;
    long long fsz;          // floats per 2-D field
    int fw, fw2;            // frame width, 2*FW
    int gx2, gx3, gy2, gy3; // reference subgrid_bounds (one rank)
    int abs_type;           // 0 none, 1 CPML, 2 damping (0 when FW == 0)
    int free_surf, boundary, L;
    int model_stride_on;    // 1: model per shot, 0: shared
    int el_tti_rb_short;    // EL_TTI CPML: right-bottom corner pass stops at NY-1
    int shot_fast;          // block index: shot varies fastest (model tiles shared in L2)
    int seismo, ndt;        // sampling (gv->SEISMO, gv->NDT)
    // TTI CPML memory of the velocity derivatives in two buffers (psi_pp = 1):
    // step n reads buffer (n - 1) & 1 and writes buffer n & 1; the second
    // buffer starts psi_xsz / psi_ysz floats after the first
    int psi_pp;
    long long psi_xsz, psi_ysz;
    int ab4;                // FDORDER_TIME = 4 (Adams-Bashforth)
    float dhi4;             // 1.0 / DH rounded to float, as the 4th-order updates compute it
    float dt, dh, dtdh, dhi, dthalbe;
    float hc[7];
    // device: time steps completed; the velocity kernel advances it. Kept last:
    // with it here the four-cell velocity kernel fits 64 registers unspilled
    int *step_ctr;
};

// Wavefield and CPML memory (per shot).
struct Wave {
    float *vx, *vy, *sxx, *syy, *sxy;
    float *r, *p, *q;                          // L planes per shot: [(s*L + l-1) * fsz]
    float *psi_sxx_x, *psi_sxy_x, *psi_vxx, *psi_vyx;  // [s][NY][2FW]
    float *psi_syy_y, *psi_sxy_y, *psi_vyy, *psi_vxy;  // [s][2FW][NX]
    float *draw, *dcor;                        // TTI: 4 derivative fields each, per shot
    // FDORDER_TIME = 4: four buffers of each history (stress-derivative sums,
    // velocity derivatives); buffer k of shot s at base + k*ab_lvl + s*fsz.
    // The memory variables then hold four levels too, ab_mlvl apart.
    float *svx4, *svy4, *hxx4, *hyy4, *hxy4, *hyx4;
    long long ab_lvl, ab_mlvl;
    // MODE = FWI forward pass (null otherwise): the velocity update writes
    // rip (sxx_x + sxy_y) / DH and rjp (sxy_x + syy_y) / DH of every cell
    // (wavefield_update_v.c:31-35) to fa_x / fa_y. On a stored step with
    // VELOCITY = 1, fstore is the store ([slots][5][NY][NX], one shot) and the
    // EL_ISO stress update writes slot nt - 1 - *fbase itself: fa_x, fa_y and
    // its u2, u3, u1 / DT (wavefield_update_s_el.c:43-47).
    float *fa_x, *fa_y;
    float *fstore;
    const int *fbase;
};

// Device state of an FWI gradient pass (sofi_fwi.cu); one shot per context.
struct FwiDev {
    float *store;                   // [slots][5][NY][NX] forward quantities of step nt in slot nt - 1 - *base
    const int *base;                // device: the step before the store's first slot (0, or a segment's start)
    float *px, *py;                 // backward, VELOCITY = 0: running sums of v * DT ([NY][NX])
    float *g_lam, *g_mu, *g_rhos;   // per-shot gradient sums ([NY][NX])
    const float *vp, *vs, *rho;     // the model as read ([NY][NX])
    double *rc;                     // [3][NY][NX]: 1 / (4 (lam+mu)^2), 1 / mu^2, 1 / (lam+mu)^2 (calc_conv.c)
    const float *adj;               // [2][ntr][NT] adjoint signals (x, y)
    const int *cell_off, *cell_rec; // receivers by cell: cell k holds cell_rec[cell_off[k] .. cell_off[k+1])
    const int *cell_map;            // [NY][NX]: k + 1 at receiver cell k, else 0
    int *bstep;                     // device: the backward step last completed (k_fwi_conv writes it)
    int ncell, ntr, nt, velocity, adjoint;
};

// Prepared model arrays (one per shot or shared) and 1-D vectors.
struct Model {
    const float *prip, *prjp;
    const float *g, *f, *fipjp;                 // isotropic (unrelaxed for visco)
    const float *db, *eb, *dipb;                // isotropic visco bases: pu*taus, pi*taup, uipjp*tausipjp
    const float *c11, *c13, *c33, *c15, *c35, *c55ipjp, *c15ipjp, *c35ipjp;   // anisotropic (DT-scaled)
    const float *c11b, *c13b, *c33b, *c15b, *c35b, *c55ipjpb, *c15ipjpb, *c35ipjpb;  // visco bases c*tau
    const float *ppi, *pu, *taus, *taup;        // surface / sampling
    const float *absorb;
    const float *K_x, *a_x, *b_x, *K_x_half, *a_x_half, *b_x_half;
    const float *K_y, *a_y, *b_y, *K_y_half, *a_y_half, *b_y_half;
    float bip[MAXL], cip[MAXL], peta[MAXL];
};

// Sources / receivers / sections of all shots (flattened with per-shot offsets).
struct Acq {
    const int *src_off;      // [nshots+1] offsets into the source arrays
    const int *src_ix, *src_iy, *src_type;
    const float *src_amp, *src_sin, *src_cos, *src_sin2, *src_cos2;  // amplitude, sin/cos(azimuth), sin/cos(2 dip)
    const float *signals;    // [total sources][nt]
    const int *last_type;    // [nshots] type of each shot's last source
    const int *rec_off;      // [nshots+1]
    const int *rec_ix, *rec_iy;
    const int *rec_col_off;  // [nshots][NX+1]: receivers of column i at rec_col_idx[off[i-1] .. off[i])
    const int *rec_col_idx;  // global receiver indices, grouped by shot and column
    float *sec;              // [total receivers][5][ns]
    int nt, ns;
    int *status;             // [nshots] 0 ok, else first unstable step
    // [nshots][NY][NX] (row-major, cell (j, i) at (j-1) NX + i-1; null unless
    // the stress kernel may do the post work): bit 0 an explosive injection of
    // the shot at the cell, bit 1 a receiver
    const unsigned char *cell_flag;
};

__device__ __forceinline__ long long cell(const Geo &G, int j, int i)
{
    return (long long)(j - 1 + HY) * G.pitch + (i - 1 + HX);
}

// Tile column and shot of this block. With a shared model and several shots
// the shot varies fastest in blockIdx.x, so the blocks that run together read
// the same model tile and only the first of them fetches it from DRAM.
// `b` is the block index.
__device__ __forceinline__ void block_xs(const Geo &G, const uint3 &b, int &bx, int &s)
{
    if (G.shot_fast) {
        s = b.x % G.nshots;
        bx = b.x / G.nshots;
    } else {
        s = b.z;
        bx = b.x;
    }
}
__device__ __forceinline__ void block_xs(const Geo &G, int &bx, int &s)
{
    block_xs(G, blockIdx, bx, s);
}

__device__ __forceinline__ long long moff(const Geo &G, int s)
{
    return G.model_stride_on ? (long long)s * G.fsz : 0;
}

// ------------------------------------------------------------ FD operators

// op_v_fdN (reference initfd.c:97-183): stress derivatives, unscaled.
template <int ND>
__device__ __forceinline__ void op_v(const float *__restrict__ sxx, const float *__restrict__ syy,
                                     const float *__restrict__ sxy, long long o, int P, const float *hc,
                                     float &sxx_x, float &sxy_x, float &sxy_y, float &syy_y)
{
    sxx_x = hc[1] * (__ldg(sxx + o + 1) - __ldg(sxx + o));
    sxy_x = hc[1] * (__ldg(sxy + o) - __ldg(sxy + o - 1));
    sxy_y = hc[1] * (__ldg(sxy + o) - __ldg(sxy + o - P));
    syy_y = hc[1] * (__ldg(syy + o + P) - __ldg(syy + o));
#pragma unroll
    for (int m = 2; m <= ND; m++) {
        sxx_x += hc[m] * (__ldg(sxx + o + m) - __ldg(sxx + o - m + 1));
        sxy_x += hc[m] * (__ldg(sxy + o + m - 1) - __ldg(sxy + o - m));
        sxy_y += hc[m] * (__ldg(sxy + o + (long long)(m - 1) * P) - __ldg(sxy + o - (long long)m * P));
        syy_y += hc[m] * (__ldg(syy + o + (long long)m * P) - __ldg(syy + o - (long long)(m - 1) * P));
    }
}

// op_s_fdN (reference initfd.c:9-95): velocity derivatives, times 1/DH.
template <int ND>
__device__ __forceinline__ void op_s(const float *__restrict__ vx, const float *__restrict__ vy, long long o,
                                     int P, const float *hc, float dhi, float &vxx, float &vyx, float &vxy,
                                     float &vyy)
{
    vxx = hc[1] * (__ldg(vx + o) - __ldg(vx + o - 1));
    vyx = hc[1] * (__ldg(vy + o + 1) - __ldg(vy + o));
    vxy = hc[1] * (__ldg(vx + o + P) - __ldg(vx + o));
    vyy = hc[1] * (__ldg(vy + o) - __ldg(vy + o - P));
#pragma unroll
    for (int m = 2; m <= ND; m++) {
        vxx += hc[m] * (__ldg(vx + o + m - 1) - __ldg(vx + o - m));
        vyx += hc[m] * (__ldg(vy + o + m) - __ldg(vy + o - m + 1));
        vxy += hc[m] * (__ldg(vx + o + (long long)m * P) - __ldg(vx + o - (long long)(m - 1) * P));
        vyy += hc[m] * (__ldg(vy + o + (long long)(m - 1) * P) - __ldg(vy + o - (long long)m * P));
    }
    vxx *= dhi;
    vyx *= dhi;
    vxy *= dhi;
    vyy *= dhi;
}

// Frame membership of column i / row j: 0 middle, 1 left/top (h = i or j),
// 2 right/bottom (h = i - NX + 2FW or j - NY + 2FW); reference update_v_PML.c.
__device__ __forceinline__ int xside(const Geo &G, int i)
{
    return i <= G.gx2 ? 1 : (i > G.gx3 ? 2 : 0);
}
__device__ __forceinline__ int yside(const Geo &G, int j)
{
    return j <= G.gy2 ? 1 : (j > G.gy3 ? 2 : 0);
}
// Region order of the reference's drivers: 0 interior, 1 left, 2 right, 3 top,
// 4 bottom, 5 left-top, 6 left-bottom, 7 right-top, 8 right-bottom.
__device__ __forceinline__ int region(const Geo &G, int i, int j)
{
    int xr = xside(G, i), yr = yside(G, j);
    if (!yr)
        return xr;
    if (!xr)
        return 2 + yr;
    return 4 + (xr - 1) * 2 + yr;
}

// CPML stretch of the four velocity derivatives of one cell (cpml_update.c:30-46
// with the drivers' h rules): memory read from R, updated memory written to Wr
// when `write` is set.
__device__ __forceinline__ void cpml_s2(const Geo &G, const Wave &R, const Wave &Wr, const Model &M, int s, int i,
                                        int j, int xr, int yr, float &vxx, float &vyx, float &vxy, float &vyy,
                                        bool write)
{
    if (xr) {
        int h = xr == 1 ? i : i - G.nx + G.fw2;
        long long q = ((long long)s * G.ny + (j - 1)) * G.fw2 + (h - 1);
        float p1 = M.b_x[h - 1] * R.psi_vxx[q] + M.a_x[h - 1] * vxx;
        vxx = vxx / M.K_x[h - 1] + p1;
        float p2 = M.b_x_half[h - 1] * R.psi_vyx[q] + M.a_x_half[h - 1] * vyx;
        vyx = vyx / M.K_x_half[h - 1] + p2;
        if (write) {
            Wr.psi_vxx[q] = p1;
            Wr.psi_vyx[q] = p2;
        }
    }
    if (yr) {
        int h = yr == 1 ? j : j - G.ny + G.fw2;
        long long q = ((long long)s * G.fw2 + (h - 1)) * G.nx + (i - 1);
        float p1 = M.b_y[h - 1] * R.psi_vyy[q] + M.a_y[h - 1] * vyy;
        vyy = vyy / M.K_y[h - 1] + p1;
        float p2 = M.b_y_half[h - 1] * R.psi_vxy[q] + M.a_y_half[h - 1] * vxy;
        vxy = vxy / M.K_y_half[h - 1] + p2;
        if (write) {
            Wr.psi_vyy[q] = p1;
            Wr.psi_vxy[q] = p2;
        }
    }
}

// The same with the memory updated in place.
__device__ __forceinline__ void cpml_s(const Geo &G, const Wave &W, const Model &M, int s, int i, int j, int xr,
                                       int yr, float &vxx, float &vyx, float &vxy, float &vyy, bool write)
{
    cpml_s2(G, W, W, M, s, i, j, xr, yr, vxx, vyx, vxy, vyy, write);
}

// Point W's velocity-derivative CPML memory at the buffer this step writes
// (previous = false) or at the one the previous step wrote (previous = true).
__device__ __forceinline__ void psi_buffers(const Geo &G, Wave &W, bool previous)
{
    if (!G.psi_pp)
        return;
    const long long b = (*G.step_ctr & 1) ^ (previous ? 1 : 0);
    W.psi_vxx += b * G.psi_xsz;
    W.psi_vyx += b * G.psi_xsz;
    W.psi_vyy += b * G.psi_ysz;
    W.psi_vxy += b * G.psi_ysz;
}

}  // namespace sofi
