// Deposit and charge-density kernels instantiated for the PCS shape (order 4), apart from
// its push kernels so that the heaviest translation units compile in parallel.
#include "kernels_push.cuh"

namespace picgb
{
    PICGB_SHAPE_LAUNCHERS(4, PCS)
} // namespace picgb
