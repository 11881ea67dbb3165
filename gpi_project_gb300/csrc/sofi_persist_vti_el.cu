// sofi_persist_vti_el.cu -- the persistent step kernel of VTI media, elastic.
#include "sofi_launch.h"
#include "sofi_persist.cuh"

namespace sofi {
template int persist_capacity_kv<VTI, false>(int, int, int);
template cudaError_t launch_persist_kv<VTI, false>(const Geo &, const Wave &, const Model &, const Acq &, int,
                                                   const PersistArgs &, int, cudaStream_t);
}
