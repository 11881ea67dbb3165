// sofi_fused_iso_el.cu -- the fused velocity + stress step of ISO media, elastic.
#include "sofi_fused.cuh"
#include "sofi_launch.h"

namespace sofi {
template void launch_fused_kv<ISO, false>(const Geo &, const Wave &, const Wave &, const Model &, int, cudaStream_t);
}
