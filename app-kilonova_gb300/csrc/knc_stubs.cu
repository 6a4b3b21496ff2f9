// Entry points of the mixed-precision stage and the learned c2p guess that
// are not built yet: they refuse with KNC_ERR_UNSUPPORTED.
#include "knc_internal.h"

namespace knc {
cudaError_t launch_c2p_mixed(const StageArgs&, cudaStream_t) { return cudaErrorNotSupported; }
cudaError_t launch_update_mixed(const StageArgs&, cudaStream_t) { return cudaErrorNotSupported; }
}  // namespace knc

extern "C" {
size_t knc_mlp_num_params(void) { return KNC_MLP_NUM_PARAMS; }
int knc_sample_pairs(knc_ctx*, int32_t, double*, int64_t, int64_t*) { return KNC_ERR_UNSUPPORTED; }
int knc_generate_pairs(double, double, double, double, double, uint64_t, int64_t, double*) {
    return KNC_ERR_UNSUPPORTED;
}
int knc_mlp_train(const double*, int64_t, float*, const knc_mlp_train_params*, float*) {
    return KNC_ERR_UNSUPPORTED;
}
int knc_mlp_forward_backward(const float*, const float*, const float*, int32_t, float*, float*, float*) {
    return KNC_ERR_UNSUPPORTED;
}
void knc_mlp_features(const double*, float*) {}
}
