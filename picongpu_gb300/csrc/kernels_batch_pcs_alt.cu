// Batched (ensemble) push kernels instantiated for the PCS shape, HigueraCary and Vay pushers, Esirkepov deposit.
#include "kernels_batch.cuh"

namespace picgb
{
    PICGB_BATCH_LAUNCHERS(4, PCSAlt, true, false)
} // namespace picgb
