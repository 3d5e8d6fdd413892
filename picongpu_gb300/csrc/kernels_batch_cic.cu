// Batched (ensemble) push kernels instantiated for the CIC shape.
#include "kernels_batch.cuh"

namespace picgb
{
    PICGB_BATCH_LAUNCHERS(1, CIC)
} // namespace picgb
