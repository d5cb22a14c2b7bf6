// tcgen05 split-precision Hankel contraction for the weighted-window moving
// averages (placeholder until the tensor-core kernel lands: reports
// NOT_IMPLEMENTED so the caller takes the FP32 CUDA-core kernel).
#include "vta_internal.h"

namespace vta {

vta_status launch_wwma_batch_tc(const WwmaBatchArgs&, int, vta_ctx*, cudaStream_t) {
    return fail(VTA_ERR_NOT_IMPLEMENTED, "tcgen05 contraction not built");
}

}  // namespace vta
