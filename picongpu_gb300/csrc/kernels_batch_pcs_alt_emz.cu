// Batched (ensemble) push kernels instantiated for the PCS shape, HigueraCary and Vay pushers, EmZ deposit.
#include "kernels_batch.cuh"

namespace picgb
{
    PICGB_BATCH_LAUNCHERS(4, PCSAltEmZ, true, true)
} // namespace picgb
