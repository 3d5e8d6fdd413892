// Push (Boris and Free; Esirkepov or EmZ), deposit and charge-density kernels
// instantiated for the TSC shape (order 2).
#include "kernels_push.cuh"

namespace picgb
{
    PICGB_PUSH_LAUNCHER(2, TSC, false)
    PICGB_SHAPE_LAUNCHERS(2, TSC)
} // namespace picgb
