// Batched (ensemble) push kernels instantiated for the PQS shape.
#include "kernels_batch.cuh"

namespace picgb
{
    PICGB_BATCH_LAUNCHERS(3, PQS)
} // namespace picgb
