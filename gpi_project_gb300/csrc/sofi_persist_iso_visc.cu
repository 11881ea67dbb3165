// sofi_persist_iso_visc.cu -- the persistent step kernel of ISO media, viscoelastic.
#include "sofi_launch.h"
#include "sofi_persist.cuh"

namespace sofi {
template int persist_capacity_kv<ISO, true>(int, int, int);
template cudaError_t launch_persist_kv<ISO, true>(const Geo &, const Wave &, const Model &, const Acq &, int,
                                                   const PersistArgs &, int, cudaStream_t);
}
