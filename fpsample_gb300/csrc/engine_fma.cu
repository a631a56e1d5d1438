// Pruned FPS engine (kd-line and vanilla, single and batched) instantiated for
// the fma floating-point mode.
#include "engine.cuh"

namespace fpsgpu {
int run_engine_fma(int dim, const EngineCall& c) { return run_engine_dispatch<true>(dim, c); }
int run_batch_fma(int dim, const BatchCall& c) { return run_batch_dispatch<true>(dim, c); }
}  // namespace fpsgpu
