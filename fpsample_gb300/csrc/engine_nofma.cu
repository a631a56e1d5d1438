// Pruned FPS engine (kd-line and vanilla, single and batched) instantiated for
// the nofma floating-point mode.
#include "engine.cuh"

namespace fpsgpu {
int run_engine_nofma(int dim, const EngineCall& c) { return run_engine_dispatch<false>(dim, c); }
int run_batch_nofma(int dim, const BatchCall& c) { return run_batch_dispatch<false>(dim, c); }
}  // namespace fpsgpu
