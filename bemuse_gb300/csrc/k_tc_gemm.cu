// k_tc_gemm.cu -- tcgen05 (TF32) trailing update of the complex LU.
#include "bem_internal.h"

namespace bem {

int tc_gemm_supported(int device) {
    (void)device;
    return 0;
}

void tc_trailing_update(cudaStream_t st, int n, int k0, int nb, CMat<float> A, const float* wl, const float* wut) {
    (void)st; (void)n; (void)k0; (void)nb; (void)A; (void)wl; (void)wut;
}

}  // namespace bem
