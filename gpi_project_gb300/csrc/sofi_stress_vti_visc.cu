// sofi_stress_vti_visc.cu -- stress kernels of VTI media, VISCO = true.
#include "sofi_stress.cuh"

namespace sofi {
template void launch_stress_kv<VTI, true>(const Geo &, const Wave &, const Model &, int, int, bool, dim3,
                                        cudaStream_t, const Acq *);
}
