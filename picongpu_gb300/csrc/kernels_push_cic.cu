// Push (Boris and Free; Esirkepov or EmZ), deposit and charge-density kernels
// instantiated for the CIC shape (order 1).
#include "kernels_push.cuh"

namespace picgb
{
    PICGB_PUSH_LAUNCHER(1, CIC, false)
    PICGB_SHAPE_LAUNCHERS(1, CIC)
} // namespace picgb
