// sofi_launch.h -- host launchers of kernels compiled in other translation units.
#pragma once
#include <cuda_runtime.h>

namespace sofi {
struct Geo;
struct Wave;
struct Model;
// velocity update, y-marching (any WEQ): rows per block `sy`
void launch_march_v(const Geo &G, const Wave &W, const Model &M, int nd, int sy, cudaStream_t st);
// stress update of isotropic / VTI media, y-marching
void launch_march_s(const Geo &G, const Wave &W, const Model &M, int nd, int kind, bool visco, int sy,
                    cudaStream_t st);
}  // namespace sofi
