// Batched (ensemble) push kernels instantiated for the CIC shape, HigueraCary and Vay pushers, EmZ deposit.
#include "kernels_batch.cuh"

namespace picgb
{
    PICGB_BATCH_LAUNCHERS(1, CICAltEmZ, true, true)
} // namespace picgb
