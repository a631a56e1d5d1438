// Vanilla FPS kernels instantiated for the nofma floating-point mode.
#include "vanilla.cuh"

namespace fpsgpu {
int run_vanilla_nofma(const VanillaCall& c) { return run_vanilla_dispatch<false>(c); }
}  // namespace fpsgpu
