// Batched (ensemble) push kernels instantiated for the PQS shape, Boris and Free pushers.
#include "kernels_batch.cuh"

namespace picgb
{
    PICGB_BATCH_LAUNCHERS(3, PQS, false)
} // namespace picgb
