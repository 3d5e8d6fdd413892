// Batched (ensemble) push kernels instantiated for the TSC shape.
#include "kernels_batch.cuh"

namespace picgb
{
    PICGB_BATCH_LAUNCHERS(2, TSC)
} // namespace picgb
