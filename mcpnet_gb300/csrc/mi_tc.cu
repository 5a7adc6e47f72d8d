// Tensor-core (tcgen05) B-spline MI: placeholder until the kernel lands.
#include "internal.h"

namespace mcpg {
cudaError_t launch_mi_tc(const uint16_t*, const uint16_t*, int64_t, const double*, int64_t, int64_t, int, int, int,
                         float*, int64_t, int*, cudaStream_t, int64_t*) {
    return cudaErrorNotSupported;
}
}  // namespace mcpg
