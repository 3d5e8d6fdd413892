// Push/deposit/charge-density kernels instantiated for the PQS shape (order 3).
#include "kernels_push.cuh"

namespace picgb
{
    PICGB_SHAPE_LAUNCHERS(3, PQS)
} // namespace picgb
