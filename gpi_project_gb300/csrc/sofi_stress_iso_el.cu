// sofi_stress_iso_el.cu -- stress kernels of ISO media, VISCO = false.
#include "sofi_stress.cuh"

namespace sofi {
template void launch_stress_kv<ISO, false>(const Geo &, const Wave &, const Model &, int, int, bool, dim3,
                                        cudaStream_t, const Acq *);
}
