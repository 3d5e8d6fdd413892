// Batched (ensemble) push kernels instantiated for the PQS shape, HigueraCary and Vay pushers, EmZ deposit.
#include "kernels_batch.cuh"

namespace picgb
{
    PICGB_BATCH_LAUNCHERS(3, PQSAltEmZ, true, true)
} // namespace picgb
