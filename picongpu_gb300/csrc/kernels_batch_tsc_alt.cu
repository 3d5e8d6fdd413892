// Batched (ensemble) push kernels instantiated for the TSC shape, HigueraCary and Vay pushers, Esirkepov deposit.
#include "kernels_batch.cuh"

namespace picgb
{
    PICGB_BATCH_LAUNCHERS(2, TSCAlt, true, false)
} // namespace picgb
