// Push kernels (Boris and Free; Esirkepov or EmZ) instantiated for the PCS shape (order 4).
#include "kernels_push.cuh"

namespace picgb
{
    PICGB_PUSH_LAUNCHER(4, PCS, false)
} // namespace picgb
