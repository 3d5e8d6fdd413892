// Batched (ensemble) push kernels instantiated for the PCS shape, Boris and Free pushers, EmZ deposit.
#include "kernels_batch.cuh"

namespace picgb
{
    PICGB_BATCH_LAUNCHERS(4, PCSEmZ, false, true)
} // namespace picgb
