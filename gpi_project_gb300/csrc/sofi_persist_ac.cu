// sofi_persist_ac.cu -- the persistent step kernel of acoustic media.
#include "sofi_launch.h"
#include "sofi_persist.cuh"

namespace sofi {
template int persist_capacity_kv<AC, false>(int, int, int);
template cudaError_t launch_persist_kv<AC, false>(const Geo &, const Wave &, const Model &, const Acq &, int,
                                                   const PersistArgs &, int, cudaStream_t);
}
