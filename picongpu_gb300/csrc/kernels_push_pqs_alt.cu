// Push kernels for the HigueraCary and Vay pushers (Esirkepov or EmZ) instantiated for
// the PQS shape (order 3).
#include "kernels_push.cuh"

namespace picgb
{
    PICGB_PUSH_LAUNCHER(3, PQSAlt, true)
} // namespace picgb
