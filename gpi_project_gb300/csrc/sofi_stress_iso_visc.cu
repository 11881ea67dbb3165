// sofi_stress_iso_visc.cu -- stress kernels of ISO media, VISCO = true.
#include "sofi_persist.cuh"
#include "sofi_stress.cuh"

namespace sofi {
template void launch_stress_kv<ISO, true>(const Geo &, const Wave &, const Model &, int, int, dim3, cudaStream_t);
template int persist_capacity_kv<ISO, true>(int, int, int);
template cudaError_t launch_persist_kv<ISO, true>(const Geo &, const Wave &, const Model &, const Acq &, int,
                                                   const PersistArgs &, int, cudaStream_t);
}
