// Batched (ensemble) push kernels instantiated for the CIC shape, Boris and Free pushers, Esirkepov deposit.
#include "kernels_batch.cuh"

namespace picgb
{
    PICGB_BATCH_LAUNCHERS(1, CIC, false, false)
} // namespace picgb
