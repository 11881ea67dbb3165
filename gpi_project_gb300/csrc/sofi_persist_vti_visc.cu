// sofi_persist_vti_visc.cu -- the persistent step kernel of VTI media, viscoelastic.
#include "sofi_launch.h"
#include "sofi_persist.cuh"

namespace sofi {
template int persist_capacity_kv<VTI, true>(int, int, int);
template cudaError_t launch_persist_kv<VTI, true>(const Geo &, const Wave &, const Model &, const Acq &, int,
                                                   const PersistArgs &, int, cudaStream_t);
}
