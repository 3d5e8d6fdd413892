// Push/deposit/charge-density kernels instantiated for the CIC shape (order 1).
#include "kernels_push.cuh"

namespace picgb
{
    PICGB_SHAPE_LAUNCHERS(1, CIC)
} // namespace picgb
