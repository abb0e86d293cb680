// Parameter gradient of sum_b coeff_b log psi^2_b (reverse mode with recomputation).
#include "net.cuh"

extern "C" int dw_log_psi_sqr_backward(const DwArch* arch, int precision, const float* params, const void* prepared,
                                       const float* r, int n_walkers, const float* R, const int32_t* Z,
                                       const float* coeff, float* grad_params, void* workspace,
                                       size_t workspace_bytes, void* stream) {
    (void)arch; (void)precision; (void)params; (void)prepared; (void)r; (void)n_walkers; (void)R; (void)Z;
    (void)coeff; (void)grad_params; (void)workspace; (void)workspace_bytes; (void)stream;
    return DW_ERR_UNSUPPORTED;
}
