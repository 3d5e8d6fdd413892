// Batched (ensemble) push kernels instantiated for the PQS shape, Boris and Free pushers, EmZ deposit.
#include "kernels_batch.cuh"

namespace picgb
{
    PICGB_BATCH_LAUNCHERS(3, PQSEmZ, false, true)
} // namespace picgb
