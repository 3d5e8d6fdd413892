// Push/deposit/charge-density kernels instantiated for the TSC shape (order 2).
#include "kernels_push.cuh"

namespace picgb
{
    PICGB_SHAPE_LAUNCHERS(2, TSC)
} // namespace picgb
