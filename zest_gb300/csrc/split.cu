// Split-precision form of the Zernike contractions (placeholder until the
// tcgen05 kernels land: reports "unsupported", never falls back).
#include "common.cuh"
#include "context.cuh"
#include "split.cuh"

namespace zgpu {

struct SplitState {};
void destroy_split(SplitState* s) { delete s; }

int split_available() { return fail(ZEST_GPU_ERR_UNSUPPORTED, "split precision is not built in this library"); }

int split_zt_forward(zest_gpu_context*, ZtPlan&, int, int, int, int, const double*, double*) {
    return split_available();
}
int split_zt_backward(zest_gpu_context*, ZtPlan&, int, int, int, int, const double*, double*) {
    return split_available();
}

}  // namespace zgpu
