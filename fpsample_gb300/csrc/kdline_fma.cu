// kd-line QuickFPS kernels instantiated for the fma floating-point mode.
#include "kdline.cuh"

namespace fpsgpu {
int run_kdline_fma(const KdlineCall& c) { return run_kdline_dispatch<true>(c); }
}  // namespace fpsgpu
