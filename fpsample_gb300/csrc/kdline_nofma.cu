// kd-line QuickFPS kernels instantiated for the nofma floating-point mode.
#include "kdline.cuh"

namespace fpsgpu {
int run_kdline_nofma(const KdlineCall& c) { return run_kdline_dispatch<false>(c); }
}  // namespace fpsgpu
