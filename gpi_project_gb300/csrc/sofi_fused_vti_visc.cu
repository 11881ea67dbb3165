// sofi_fused_vti_visc.cu -- the fused velocity + stress step of VTI media, viscoelastic.
#include "sofi_fused.cuh"
#include "sofi_launch.h"

namespace sofi {
template void launch_fused_kv<VTI, true>(const Geo &, const Wave &, const Wave &, const Model &, int, cudaStream_t);
}
