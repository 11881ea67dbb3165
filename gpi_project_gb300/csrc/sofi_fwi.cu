// sofi_fwi.cu -- the FWI gradient pass of one shot (MODE = FWI, EL_ISO) on
// the device: inversion.c's forward run with snap_store.c, its backward run
// with the residuals injected at the receivers (update_v_interior.c:72-90) and
// calc_conv.c's correlation at every step (time_loop.c:288-303, DTINV = 1).
//
// Forward: the store holds [slots][5][NY][NX] floats, slot nt - 1 when the
// whole run is kept, slot nt - 1 - base for a recomputed segment of a
// checkpointed pass (base = the segment's first step - 1). The velocity
// kernel writes this step's rip / rjp terms (Wave::fa_*); with VELOCITY = 1
// the stress kernel then fills the whole slot (those two and its own u / DT),
// with VELOCITY = 0 k_fwi_store copies them and the stresses after the free
// surface.
// Backward, per step: the velocity kernel (k_update_vw_bwd) adds the adjoint
// signals at the receivers before its update, forms the reference's pvxp1 /
// pvyp1 (the injected velocity, or its running sum times DT for VELOCITY =
// 0) and adds the density term; after the stress update and the free surface
// k_fwi_conv adds the lambda and mu terms against forward slot NT - nt + 1
// and records the step it completed (FwiDev::bstep) for the next velocity
// kernel, which advances the step counter while its blocks run.
// Every kernel takes the step number from the device counter, so the steps
// replay from the captured graph like the plain ones; the per-step kernels
// are launched as programmatic dependents (pdl_begin) like the step's own.
#include "sofi_common.cuh"
#include "sofi_launch.h"

namespace sofi {

// VELOCITY = 0 only
__global__ void k_fwi_store(Geo G, Wave W, FwiDev F)
{
    pdl_begin();
    const long long n = (long long)G.nx * G.ny;
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n)
        return;
    const int nt = *G.step_ctr;  // the step just completed
    const int j = (int)(q / G.nx) + 1, i = (int)(q % G.nx) + 1;
    const long long o = cell(G, j, i);
    float *slot = F.store + (long long)(nt - 1 - *F.base) * 5 * n + q;
    slot[0] = W.fa_x[o];
    slot[n] = W.fa_y[o];
    slot[2 * n] = W.sxx[o], slot[3 * n] = W.syy[o], slot[4 * n] = W.sxy[o];
}

// The model-only divisors of calc_conv.c:42-67, once per pass: muss / lamss
// are floats and the constants double there, so 1 / (4 (lamss + muss)^2) is
// formed in double; 1 / muss^2 and 1 / (lamss + muss)^2 are the double
// reciprocals of the float squares the reference divides by.
__global__ void k_fwi_coef(int n, FwiDev F)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n)
        return;
    const float vs0 = F.vs[q], vp0 = F.vp[q], rho0 = F.rho[q];
    const float muss = __fmul_rn(__fmul_rn(vs0, vs0), rho0);
    const float lamss = (float)__dadd_rn((double)__fmul_rn(__fmul_rn(vp0, vp0), rho0), -2.0 * (double)muss);
    const float lm = __fadd_rn(lamss, muss);
    F.rc[q] = 1.0 / __dmul_rn(__dmul_rn(4.0, (double)lm), (double)lm);
    F.rc[n + q] = 1.0 / (double)__fmul_rn(muss, muss);
    F.rc[2 * n + q] = 1.0 / (double)__fmul_rn(lm, lm);
}

// calc_conv.c:34-71: the lambda and mu terms are formed in double and rounded
// into the float sums. The reference divides by (lamss + muss)^2 and muss^2;
// here their double reciprocals multiply (at most one double ulp apart
// before the rounding to float).
__global__ void k_fwi_conv(Geo G, Wave W, Model M, FwiDev F)
{
    pdl_begin();
    const long long n = (long long)G.nx * G.ny;
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nt = *G.step_ctr;
    if (q == 0)
        *F.bstep = nt;
    if (q >= n)
        return;
    const int j = (int)(q / G.nx) + 1, i = (int)(q % G.nx) + 1;
    const long long o = cell(G, j, i);
    const float *slot = F.store + (long long)(F.nt - nt - *F.base) * 5 * n + q;
    const float fx = slot[2 * n], fy = slot[3 * n], fu = slot[4 * n];
    const float sxx = W.sxx[o], syy = W.syy[o], sxy = W.sxy[o];
    const double mDT = -(double)G.dt;
    const float sum_f = __fmul_rn(__fadd_rn(fx, fy), __fadd_rn(sxx, syy));
    F.g_lam[q] = (float)__dadd_rn((double)F.g_lam[q], __dmul_rn(__dmul_rn(mDT, F.rc[q]), (double)sum_f));
    if (M.pu[o] > 0.0f) {
        const double r_mm = F.rc[n + q], r_lm2 = F.rc[2 * n + q];
        const double t1 = __dmul_rn(r_mm, (double)__fmul_rn(fu, sxy));
        const double t2 = __dmul_rn(__dmul_rn(0.25, (double)sum_f), r_lm2);
        const double t3 = __dmul_rn(__dmul_rn(0.25, (double)__fmul_rn(__fsub_rn(fx, fy), __fsub_rn(sxx, syy))), r_mm);
        F.g_mu[q] = (float)__dadd_rn((double)F.g_mu[q], __dmul_rn(mDT, __dadd_rn(__dadd_rn(t1, t2), t3)));
    }
}

void launch_fwi_coef(int n, const FwiDev &F, cudaStream_t st)
{
    k_fwi_coef<<<(n + 255) / 256, 256, 0, st>>>(n, F);
}

void launch_fwi_store(const Geo &G, const Wave &W, const FwiDev &F, cudaStream_t st)
{
    const long long n = (long long)G.nx * G.ny;
    launch_pdl(k_fwi_store, (unsigned)((n + 255) / 256), 256, 0, st, G, W, F);
}

void launch_fwi_conv(const Geo &G, const Wave &W, const Model &M, const FwiDev &F, cudaStream_t st)
{
    const long long n = (long long)G.nx * G.ny;
    launch_pdl(k_fwi_conv, (unsigned)((n + 255) / 256), 256, 0, st, G, W, M, F);
}

}  // namespace sofi
