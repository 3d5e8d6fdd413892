// Push kernels for the HigueraCary and Vay pushers (Esirkepov or EmZ) instantiated for
// the CIC shape (order 1).
#include "kernels_push.cuh"

namespace picgb
{
    PICGB_PUSH_LAUNCHER(1, CICAlt, true)
} // namespace picgb
