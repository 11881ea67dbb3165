// sofi_stress_iso_visc.cu -- stress kernels of ISO media, VISCO = true.
#include "sofi_stress.cuh"

namespace sofi {
template void launch_stress_kv<ISO, true>(const Geo &, const Wave &, const Model &, int, int, bool, dim3,
                                        cudaStream_t, const Acq *);
}
