// Batched (ensemble) push kernels instantiated for the PQS shape, Boris and Free pushers, Esirkepov deposit.
#include "kernels_batch.cuh"

namespace picgb
{
    PICGB_BATCH_LAUNCHERS(3, PQS, false, false)
} // namespace picgb
