// Learned-proposal kernels on the tcgen05 tensor cores (see esp_lp_tc.cuh):
//
//   k_lp_forward_tc   the network over rows of features (checks)
//   k_sweep_lp_tc     one colour class of the learned Metropolis-Hastings
//                     sweep, 128 (site, replica) trials per CTA and network
//                     pass, one thread per trial
//
// The trial, its density ratio and the bookkeeping are those of k_sweep_lp
// (esp_learned.cu); only the network evaluation moves to tcgen05.
#include "esp_lp_tc.h"

namespace esp {

namespace {

__global__ void __launch_bounds__(kTcRows) k_lp_forward_tc(const LpWeights w, const __nv_bfloat16 *x, int n,
                                                            float *out, int *err, int force_timeout)
{
    extern __shared__ __align__(128) unsigned char smem[];
    TcSmem &s = *reinterpret_cast<TcSmem *>(smem);
    tc_stage_weights(w, s);
    tc_setup(s);
    uint32_t phase = 0;
    bool pending = false;
    const int t = threadIdx.x;
    for (int base = blockIdx.x * kTcRows; base < n; base += gridDim.x * kTcRows) {
        const int i = base + t;
        uint4 v0 = make_uint4(0u, 0u, 0u, 0u), v1 = v0;
        if (i < n) {
            v0 = reinterpret_cast<const uint4 *>(x + (size_t)i * kMlpInPad)[0];
            v1 = reinterpret_cast<const uint4 *>(x + (size_t)i * kMlpInPad)[1];
        }
        unsigned char *xb = reinterpret_cast<unsigned char *>(s.t[0].x);
        *reinterpret_cast<uint4 *>(xb + kmajor_offset(t, 0, kMlpInPad)) = v0;
        *reinterpret_cast<uint4 *>(xb + kmajor_offset(t, 8, kMlpInPad)) = v1;
        float o[kMlpOut];
        if (!tc_forward(s, 0, phase, o, force_timeout, pending)) break;   // the CTA's one group: uniform
        if (i < n)
            for (int k = 0; k < kMlpOut; ++k) out[(size_t)i * kMlpOut + k] = o[k];
    }
    tc_teardown(s, 0, pending, phase);
    if (t == 0 && s.error) atomicExch(err, 1);
}

}  // namespace

size_t lp_tc_smem_bytes() { return sizeof(TcSmem); }

cudaError_t lp_tc_configure()
{
    return cudaFuncSetAttribute(k_lp_forward_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TcSmem));
}

cudaError_t launch_lp_forward_tc(const LpWeights &w, const __nv_bfloat16 *x, int n, float *out, int *err,
                                 int num_sms, cudaStream_t st, int force_timeout)
{
    if (n <= 0) return cudaSuccess;
    int blocks = (n + kTcRows - 1) / kTcRows;
    if (blocks > 2 * num_sms) blocks = 2 * num_sms;
    k_lp_forward_tc<<<blocks, kTcRows, sizeof(TcSmem), st>>>(w, x, n, out, err, force_timeout);
    return cudaGetLastError();
}

}  // namespace esp
