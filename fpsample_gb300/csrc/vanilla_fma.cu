// Vanilla FPS kernels instantiated for the fma floating-point mode.
#include "vanilla.cuh"

namespace fpsgpu {
int run_vanilla_fma(const VanillaCall& c) { return run_vanilla_dispatch<true>(c); }
}  // namespace fpsgpu
