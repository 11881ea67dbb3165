// sofi_march.cu -- instantiations and launchers of the y-marching kernels
// (sofi_march.cuh), kept in their own translation unit so they compile in
// parallel with sofigpu.cu.
#include "sofi_march.cuh"
#include "sofi_launch.h"

namespace sofi {

constexpr int kTX = 128;

#define ND_CASES(ND_, ...)                                          \
    switch (ND_) {                                                  \
      case 1: { constexpr int ND = 1; __VA_ARGS__; } break;         \
      case 2: { constexpr int ND = 2; __VA_ARGS__; } break;         \
      case 3: { constexpr int ND = 3; __VA_ARGS__; } break;         \
      case 4: { constexpr int ND = 4; __VA_ARGS__; } break;         \
      case 5: { constexpr int ND = 5; __VA_ARGS__; } break;         \
      case 6: { constexpr int ND = 6; __VA_ARGS__; } break;         \
    }

static dim3 march_grid(const Geo &G, int sy)
{
    return dim3((G.nx + kTX - 1) / kTX, (G.ny + sy - 1) / sy, G.nshots);
}

void launch_march_v(const Geo &G, const Wave &W, const Model &M, int nd, int sy, cudaStream_t st)
{
    dim3 g = march_grid(G, sy);
    ND_CASES(nd, (k_march_v<ND, kTX><<<g, kTX, 0, st>>>(G, W, M, sy)));
}

template <int KIND, bool VISCO>
static void march_s_l(const Geo &G, const Wave &W, const Model &M, int nd, int sy, cudaStream_t st)
{
    dim3 g = march_grid(G, sy);
    int L = VISCO ? G.L : 0;
    if (!VISCO)
        ND_CASES(nd, (k_march_s<ND, kTX, KIND, false, 0><<<g, kTX, 0, st>>>(G, W, M, sy)))
    else if (L == 1)
        ND_CASES(nd, (k_march_s<ND, kTX, KIND, true, 1><<<g, kTX, 0, st>>>(G, W, M, sy)))
    else if (L == 2)
        ND_CASES(nd, (k_march_s<ND, kTX, KIND, true, 2><<<g, kTX, 0, st>>>(G, W, M, sy)))
    else if (L == 3)
        ND_CASES(nd, (k_march_s<ND, kTX, KIND, true, 3><<<g, kTX, 0, st>>>(G, W, M, sy)))
    else
        ND_CASES(nd, (k_march_s<ND, kTX, KIND, true, 0><<<g, kTX, 0, st>>>(G, W, M, sy)))
}

void launch_march_s(const Geo &G, const Wave &W, const Model &M, int nd, int kind, bool visco, int sy,
                    cudaStream_t st)
{
    if (kind == ISO)
        visco ? march_s_l<ISO, true>(G, W, M, nd, sy, st) : march_s_l<ISO, false>(G, W, M, nd, sy, st);
    else
        visco ? march_s_l<VTI, true>(G, W, M, nd, sy, st) : march_s_l<VTI, false>(G, W, M, nd, sy, st);
}

}  // namespace sofi
