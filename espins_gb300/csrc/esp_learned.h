// Launchers of the learned-proposal kernels (esp_learned.cu); host-side only.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "esp_device.cuh"
#include "esp_mlp.cuh"

namespace esp {

// Padded parameter block (fp32 master copy, gradients, Adam moments):
// W1 [128][16] | b1 [128] | W2 [128][128] | b2 [128] | W3 [32][128] | b3 [32]
constexpr int kPadW1 = 0;
constexpr int kPadB1 = kPadW1 + kMlpHid * kMlpInPad;
constexpr int kPadW2 = kPadB1 + kMlpHid;
constexpr int kPadB2 = kPadW2 + kMlpHid * kMlpHid;
constexpr int kPadW3 = kPadB2 + kMlpHid;
constexpr int kPadB3 = kPadW3 + kMlpOutPad * kMlpHid;
constexpr int kPadParams = kPadB3 + kMlpOutPad;

// Reference axis of the local frame per atom: the single-ion axis, or null
// for x.
struct LpSweepArgs {
    SweepArgs s;
    LpWeights w;
    const float4 *axis;   // [num_atoms] or null
    // test hook of the tcgen05 engine: every group reports a completion wait
    // that gave up after its first layer's MMAs completed (0: off)
    int tc_force_timeout;
};

struct LpCollectArgs {
    SweepArgs s;          // tables and state; off_c/n_c the colour class
    const float4 *axis;
    __nv_bfloat16 *x;     // [n][16] features (bf16, zero padded)
    float *t;             // [n][4]: unit spin in the local frame, kappa0
    long long first, count;   // write items [0, count) of the class at rows first..
};

struct GemmArgs {
    const __nv_bfloat16 *A;
    const __nv_bfloat16 *B;
    int lda, ldb, M, N, K;
    float *C;             // fp32 output or null
    int ldc, accumulate;
    __nv_bfloat16 *Cb;    // bf16 output or null
    int ldcb;
    const float *bias;    // [N] or null
    int relu;
    const __nv_bfloat16 *mask;  // multiply by (mask > 0), same shape as the output, or null
    int ldm;
};

size_t lp_sweep_smem_bytes();
int lp_sweep_blocks(long long max_items, int R, int num_sms);
cudaError_t lp_configure(int device);
cudaError_t launch_sweep_lp(const LpSweepArgs &a, bool hb, bool hd, int blocks, cudaStream_t st);
// tcgen05 variant: 128-thread CTAs with their own partial slots [blocks][slots]
// (slots = min(R, 128)); err is set when a tensor-core wait gave up
int lp_tc_sweep_blocks(long long max_items, int R, int num_sms);
cudaError_t lp_tc_sweep_configure();
cudaError_t launch_sweep_lp_tc(const LpSweepArgs &a, bool hb, bool hd, int blocks, double *part,
                               unsigned long long *part_rej, int slots, int *err, cudaStream_t st);
cudaError_t launch_lp_collect(const LpCollectArgs &a, bool hb, bool hd, int max_blocks, cudaStream_t st);
// C = op(A) op(B): ta -> A stored [K][M] (else [M][K]); tb -> B stored [K][N] (else [N][K])
cudaError_t launch_gemm(const GemmArgs &g, bool ta, bool tb, cudaStream_t st);
// The same GEMM on the tcgen05 tensor cores (esp_gemm_tc.cu): 128-row tiles
// with tensor-memory accumulators; M, K multiples of 8, N of 16.  Pure FP32
// outputs (no bias, ReLU, mask, BF16 copy or accumulation) with M*N at most
// kGemmTcSplitMN are split along K into `work` (kGemmTcMaxSplit * M * N
// floats) and summed in a fixed order.  err is set when a completion wait
// gave up.
constexpr int kGemmTcMaxSplit = 64;
constexpr int kGemmTcSplitMN = 128 * 128;
constexpr size_t kGemmTcWorkFloats = (size_t)kGemmTcMaxSplit * kGemmTcSplitMN;
cudaError_t gemm_tc_configure();
cudaError_t launch_gemm_tc(const GemmArgs &g, bool ta, bool tb, int num_sms, float *work, int *err, cudaStream_t st);
cudaError_t launch_lp_gather(const __nv_bfloat16 *x_all, const float *t_all, long long n_all, int batch,
                             uint64_t seed, uint64_t step, __nv_bfloat16 *xb, float *tb, cudaStream_t st);
// rows >= n_real of the n_rows in the batch get zero gradients and no loss
cudaError_t launch_lp_head(const float *o, const float *t, int n_real, int n_rows, float scale, __nv_bfloat16 *d_o,
                           double *loss, cudaStream_t st);
cudaError_t launch_colsum(const __nv_bfloat16 *x, int rows, int cols, int ld, float *out, cudaStream_t st);
cudaError_t launch_adam(float *p, const float *g, float *m, float *v, int n, float lr, float b1, float b2, float eps,
                        long long t, cudaStream_t st);
cudaError_t launch_lp_to_bf16(const float *p, __nv_bfloat16 *w1, __nv_bfloat16 *w2, __nv_bfloat16 *w3,
                              cudaStream_t st);
cudaError_t launch_lp_forward(const LpWeights &w, const __nv_bfloat16 *x, int n, float *out, cudaStream_t st);

}  // namespace esp
