// Batched (ensemble) push kernels instantiated for the PQS shape, HigueraCary and Vay pushers.
#include "kernels_batch.cuh"

namespace picgb
{
    PICGB_BATCH_LAUNCHERS(3, PQSAlt, true)
} // namespace picgb
