// Batched (ensemble) push kernels instantiated for the CIC shape, HigueraCary and Vay pushers, Esirkepov deposit.
#include "kernels_batch.cuh"

namespace picgb
{
    PICGB_BATCH_LAUNCHERS(1, CICAlt, true, false)
} // namespace picgb
