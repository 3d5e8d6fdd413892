// Batched (ensemble) push kernels instantiated for the PQS shape, HigueraCary and Vay pushers, Esirkepov deposit.
#include "kernels_batch.cuh"

namespace picgb
{
    PICGB_BATCH_LAUNCHERS(3, PQSAlt, true, false)
} // namespace picgb
