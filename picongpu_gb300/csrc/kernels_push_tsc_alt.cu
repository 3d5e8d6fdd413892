// Push kernels for the HigueraCary and Vay pushers (Esirkepov or EmZ) instantiated for
// the TSC shape (order 2).
#include "kernels_push.cuh"

namespace picgb
{
    PICGB_PUSH_LAUNCHER(2, TSCAlt, true)
} // namespace picgb
