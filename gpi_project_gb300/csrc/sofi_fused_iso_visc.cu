// sofi_fused_iso_visc.cu -- the fused velocity + stress step of ISO media, viscoelastic.
#include "sofi_fused.cuh"
#include "sofi_launch.h"

namespace sofi {
template void launch_fused_kv<ISO, true>(const Geo &, const Wave &, const Wave &, const Model &, int, cudaStream_t);
}
