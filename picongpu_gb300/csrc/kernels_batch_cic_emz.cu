// Batched (ensemble) push kernels instantiated for the CIC shape, Boris and Free pushers, EmZ deposit.
#include "kernels_batch.cuh"

namespace picgb
{
    PICGB_BATCH_LAUNCHERS(1, CICEmZ, false, true)
} // namespace picgb
