// Batched (ensemble) push kernels instantiated for the TSC shape, Boris and Free pushers, Esirkepov deposit.
#include "kernels_batch.cuh"

namespace picgb
{
    PICGB_BATCH_LAUNCHERS(2, TSC, false, false)
} // namespace picgb
