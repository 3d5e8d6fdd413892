// Push kernels for the HigueraCary and Vay pushers (Esirkepov or EmZ) instantiated for
// the PCS shape (order 4).
#include "kernels_push.cuh"

namespace picgb
{
    PICGB_PUSH_LAUNCHER(4, PCSAlt, true)
} // namespace picgb
