// sofi_dispatch.cuh -- run a statement with the FD half-order ND (1..6) as a
// compile-time constant.
#pragma once

#define DISPATCH_ND(ND_, ...)                                       \
    switch (ND_) {                                                  \
      case 1: { constexpr int ND = 1; __VA_ARGS__; } break;         \
      case 2: { constexpr int ND = 2; __VA_ARGS__; } break;         \
      case 3: { constexpr int ND = 3; __VA_ARGS__; } break;         \
      case 4: { constexpr int ND = 4; __VA_ARGS__; } break;         \
      case 5: { constexpr int ND = 5; __VA_ARGS__; } break;         \
      case 6: { constexpr int ND = 6; __VA_ARGS__; } break;         \
    }
