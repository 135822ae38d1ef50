// Launchers of the tcgen05 learned-proposal kernels (esp_lp_tc.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "esp_learned.h"
#include "esp_lp_tc.cuh"

namespace esp {

size_t lp_tc_smem_bytes();
cudaError_t lp_tc_configure();
// err: device int set to 1 when a tensor-core completion wait gave up;
// force_timeout (test hook): report a give-up after the first layer's MMAs
cudaError_t launch_lp_forward_tc(const LpWeights &w, const __nv_bfloat16 *x, int n, float *out, int *err,
                                 int num_sms, cudaStream_t st, int force_timeout);

}  // namespace esp
