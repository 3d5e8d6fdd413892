// Batched (ensemble) push kernels instantiated for the TSC shape, Boris and Free pushers, EmZ deposit.
#include "kernels_batch.cuh"

namespace picgb
{
    PICGB_BATCH_LAUNCHERS(2, TSCEmZ, false, true)
} // namespace picgb
