// Fused four-layer forward pass of the drainage surrogate on the tcgen05 tensor cores.
#include "nn.cuh"
#include "nn_kernels.h"
#include "sbs_internal.h"

namespace sbs {
namespace nn {

int fused_forward(sbs_surrogate *, const Fields &, int, const GridTab &, float *, size_t, float *) {
    return set_error(SBS_E_INVALID, "SBS_NN_FUSED is not available in this build");
}
int fused_pack(sbs_surrogate *) { return SBS_OK; }
void fused_release(sbs_surrogate *) {}

}  // namespace nn
}  // namespace sbs
