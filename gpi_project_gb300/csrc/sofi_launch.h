// sofi_launch.h -- host launchers of kernels compiled in other translation
// units (so that the template instantiations compile in parallel).
#pragma once
#include <cuda_runtime.h>

namespace sofi {
struct Geo;
struct Wave;
struct Model;
struct Acq;
struct FwiDev;
// FWI gradient pass (sofi_fwi.cu): forward storage after a step; the lambda /
// mu terms after the post kernel (the adjoint injection and the density term
// are part of the backward steps' velocity kernel)
void launch_fwi_coef(int n, const FwiDev &F, cudaStream_t st);  // the model-only divisors, once per pass
void launch_fwi_store(const Geo &G, const Wave &W, const FwiDev &F, cudaStream_t st);
void launch_fwi_conv(const Geo &G, const Wave &W, const Model &M, const FwiDev &F, cudaStream_t st);
// velocity update: vw cells per thread in x (4 or 2), else vrows rows per thread (1, 2, 4);
// narrow (vw 4, not acoustic): blocks of 8 x 32 threads, 32 columns by 32 rows (grid sized for that);
// acoustic: no sxy terms, vw 4, 2 or else one cell per thread;
// bwd (a backward step of an FWI pass): also the adjoint injection and the
// density term, vw 4, 2 or else one cell per thread, wide blocks
void launch_velocity(const Geo &G, const Wave &W, const Model &M, int nd, int vw, int vrows, bool narrow, bool acoustic,
                     dim3 grid, cudaStream_t st, const FwiDev *bwd = nullptr);
// Where the narrow four-cell blocks (8 x 32 threads, 32 columns by 32 rows)
// exist: the velocity update of non-acoustic media and the ISO / VTI stress
// update of elastic media or L <= 3, neither on an FWI forward step. The
// launchers and the grids they are given both follow these.
inline bool narrow_v_applies(bool acoustic, bool fwi_step)
{
    return !acoustic && !fwi_step;
}
inline bool narrow_s_applies(bool visco, int L, bool fwi_step)
{
    return !fwi_step && (!visco || (L >= 1 && L <= 3));
}
// ISO / VTI stress update (KIND 0 ISO, 1 VTI): sw cells per thread in x (4, 2 or 0 = one);
// narrow (sw 4, where narrow_s_applies): blocks of 8 x 32 threads; post (sw 0 only, else
// null): the one-cell kernel also does k_post's work with that acquisition
template <int KIND, bool VISCO>
void launch_stress_kv(const Geo &G, const Wave &W, const Model &M, int nd, int sw, bool narrow, dim3 grid,
                      cudaStream_t st, const Acq *post = nullptr);
// A backward step of an FWI pass (EL_ISO) without a free surface: the stress
// update with the lambda / mu correlation, sw cells per thread in x (4, 2 or
// 0 = one), wide blocks; post (sw 0 only, else null): the one-cell kernel
// also does k_post's work with that acquisition
void launch_stress_bwd(const Geo &G, const Wave &W, const Model &M, const FwiDev &F, int nd, int sw, dim3 grid,
                       cudaStream_t st, const Acq *post = nullptr);
// acoustic stress update: sw cells per thread in x (4, 2 or 0/1 = one)
void launch_stress_ac(const Geo &G, const Wave &W, const Model &M, int nd, int sw, dim3 grid, cudaStream_t st);
// FDORDER_TIME = 4: step counter, velocity update, stress update (one cell per thread)
void launch_ab4_begin(const Geo &G, cudaStream_t st);
// 4th-order time stepping: `wide` four cells per thread in x (own grid), else
// one cell per thread on `grid`
void launch_ab4_v(const Geo &G, const Wave &W, const Model &M, int nd, bool wide, dim3 grid, cudaStream_t st);
void launch_ab4_s(const Geo &G, const Wave &W, const Model &M, int nd, bool visco, bool wide, dim3 grid,
                  cudaStream_t st);
// TTI stress update: one pass (derivatives in shared memory) or the two-kernel
// form (derivative fields in W.draw / W.dcor)
void launch_tti_fused(const Geo &G, const Wave &W, const Model &M, int nd, bool visco, bool cpml, dim3 grid,
                      cudaStream_t st);
void launch_tti_split(const Geo &G, const Wave &W, const Model &M, int nd, bool visco, dim3 grid, cudaStream_t st);
// the one-pass form on 32 x 8 tiles in the frame, 64 x 32 four-cell tiles elsewhere (own grid)
void launch_tti_tiles(const Geo &G, const Wave &W, const Model &M, int nd, bool visco, bool cpml, cudaStream_t st);
}  // namespace sofi
