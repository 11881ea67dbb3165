// sofi_stress_vti_el.cu -- stress kernels of VTI media, VISCO = false.
#include "sofi_stress.cuh"

namespace sofi {
template void launch_stress_kv<VTI, false>(const Geo &, const Wave &, const Model &, int, int, bool, dim3,
                                        cudaStream_t, const Acq *);
}
