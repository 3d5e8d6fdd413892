// Push (Boris and Free; Esirkepov or EmZ), deposit and charge-density kernels
// instantiated for the PQS shape (order 3).
#include "kernels_push.cuh"

namespace picgb
{
    PICGB_PUSH_LAUNCHER(3, PQS, false)
    PICGB_SHAPE_LAUNCHERS(3, PQS)
} // namespace picgb
