// Batched (ensemble) push kernels instantiated for the TSC shape, HigueraCary and Vay pushers, EmZ deposit.
#include "kernels_batch.cuh"

namespace picgb
{
    PICGB_BATCH_LAUNCHERS(2, TSCAltEmZ, true, true)
} // namespace picgb
