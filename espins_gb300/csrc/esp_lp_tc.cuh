// The learned proposal's MLP (12 -> 128 -> 128 -> 20, ReLU) on the tcgen05
// tensor cores for 128 rows at a time: one CTA of 128 threads, thread t owns
// row t (its tensor-memory lane).  Operands in shared memory in the K-major
// no-swizzle layout of esp_tc.cuh, accumulators in 128 tensor-memory columns,
// one thread issues the MMAs and an mbarrier signals their completion.
#pragma once
#include <cuda_bf16.h>

#include "esp_mlp.cuh"
#include "esp_tc.cuh"

namespace esp {

constexpr int kTcRows = 128;
constexpr uint32_t kTcCols = 128;           // tensor-memory columns per CTA
constexpr uint32_t kTcWaitLimit = 1u << 24; // mbarrier polls before giving up

struct TcSmem {
    __nv_bfloat16 w1[kMlpHid * kMlpInPad];     // [128][16] K-major
    __nv_bfloat16 w2[kMlpHid * kMlpHid];       // [128][128]
    __nv_bfloat16 w3[kMlpOutPad * kMlpHid];    // [32][128]
    __nv_bfloat16 x[kTcRows * kMlpInPad];      // [128][16]
    __nv_bfloat16 h[kTcRows * kMlpHid];        // [128][128]
    float b1[kMlpHid], b2[kMlpHid], b3[kMlpOutPad];
    unsigned long long bar;
    uint32_t tmem;
    int error;
};

// Row-major global weights ([out][in]) to the K-major operand layout.
__device__ __forceinline__ void tc_stage_weights(const LpWeights &w, TcSmem &s)
{
    auto stage = [&](const __nv_bfloat16 *src, __nv_bfloat16 *dst, int rows, int K) {
        const int chunks = rows * (K / 8);
        for (int i = threadIdx.x; i < chunks; i += blockDim.x) {
            const int r = i / (K / 8), k = (i % (K / 8)) * 8;
            const uint4 v = __ldg(reinterpret_cast<const uint4 *>(src + (size_t)r * K + k));
            *reinterpret_cast<uint4 *>(reinterpret_cast<unsigned char *>(dst) + kmajor_offset(r, k, K)) = v;
        }
    };
    stage(w.w1, s.w1, kMlpHid, kMlpInPad);
    stage(w.w2, s.w2, kMlpHid, kMlpHid);
    stage(w.w3, s.w3, kMlpOutPad, kMlpHid);
    for (int i = threadIdx.x; i < kMlpHid; i += blockDim.x) { s.b1[i] = __ldg(w.b1 + i); s.b2[i] = __ldg(w.b2 + i); }
    for (int i = threadIdx.x; i < kMlpOutPad; i += blockDim.x) s.b3[i] = __ldg(w.b3 + i);
}

// Set-up by the whole CTA: mbarrier, 128 tensor-memory columns (warp 0).
__device__ __forceinline__ void tc_setup(TcSmem &s)
{
    if (threadIdx.x == 0) {
        mbar_init(smem_u32(&s.bar), 1);
        s.error = 0;
    }
    if (threadIdx.x < 32) {
        tmem_alloc(smem_u32(&s.tmem), kTcCols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
}

__device__ __forceinline__ void tc_teardown(TcSmem &s)
{
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (threadIdx.x < 32) tmem_dealloc(s.tmem, kTcCols);
}

// Thread t's 12 features as row t of the X operand (zero padding to 16).
__device__ __forceinline__ void tc_store_x_row(TcSmem &s, int t, const float *f)
{
    uint4 v0, v1;
    v0.x = pack_bf16(f[0], f[1]); v0.y = pack_bf16(f[2], f[3]); v0.z = pack_bf16(f[4], f[5]); v0.w = pack_bf16(f[6], f[7]);
    v1.x = pack_bf16(f[8], f[9]); v1.y = pack_bf16(f[10], f[11]); v1.z = 0u; v1.w = 0u;
    unsigned char *b = reinterpret_cast<unsigned char *>(s.x);
    *reinterpret_cast<uint4 *>(b + kmajor_offset(t, 0, kMlpInPad)) = v0;
    *reinterpret_cast<uint4 *>(b + kmajor_offset(t, 8, kMlpInPad)) = v1;
}

// Issue (thread 0) the MMAs of one layer, commit, and wait (every thread).
// Returns false when the wait gave up.
__device__ __forceinline__ bool tc_layer(TcSmem &s, const __nv_bfloat16 *a, int K, const __nv_bfloat16 *b, int N,
                                         uint32_t &phase)
{
    fence_async_smem();     // this thread's operand writes -> tensor cores
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (threadIdx.x == 0) {
        const uint32_t idesc = idesc_bf16_f32(kTcRows, N);
        const uint32_t sbo = (uint32_t)(K / 8) * 128u;
        const uint32_t a0 = smem_u32(a), b0 = smem_u32(b);
        for (int kk = 0; kk < K / 16; ++kk)
            tc_mma(s.tmem, smem_desc(a0 + 256u * kk, 128u, sbo), smem_desc(b0 + 256u * kk, 128u, sbo), idesc, kk > 0);
        tc_commit(smem_u32(&s.bar));
    }
    const bool ok = mbar_wait(smem_u32(&s.bar), phase, kTcWaitLimit);
    phase ^= 1u;
    tc_fence_after();
    if (!ok) s.error = 1;
    return ok;
}

// Hidden-layer epilogue: relu(D + bias) of this thread's row to H.
__device__ __forceinline__ void tc_hidden_epilogue(TcSmem &s, const float *bias)
{
    const int t = threadIdx.x;
    const uint32_t lane_base = s.tmem + ((uint32_t)(t & ~31) << 16);
    unsigned char *hb = reinterpret_cast<unsigned char *>(s.h);
#pragma unroll 1
    for (int c0 = 0; c0 < kMlpHid; c0 += 16) {
        float v[16];
        tmem_ld16(lane_base + (uint32_t)c0, v);
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            uint4 p;
            const int c = c0 + 8 * half;
            p.x = pack_bf16(fmaxf(v[8 * half + 0] + bias[c + 0], 0.f), fmaxf(v[8 * half + 1] + bias[c + 1], 0.f));
            p.y = pack_bf16(fmaxf(v[8 * half + 2] + bias[c + 2], 0.f), fmaxf(v[8 * half + 3] + bias[c + 3], 0.f));
            p.z = pack_bf16(fmaxf(v[8 * half + 4] + bias[c + 4], 0.f), fmaxf(v[8 * half + 5] + bias[c + 5], 0.f));
            p.w = pack_bf16(fmaxf(v[8 * half + 6] + bias[c + 6], 0.f), fmaxf(v[8 * half + 7] + bias[c + 7], 0.f));
            *reinterpret_cast<uint4 *>(hb + kmajor_offset(t, c, kMlpHid)) = p;
        }
    }
}

// The whole network for the 128 rows of s.x; thread t gets row t's 20
// outputs.  Returns false if a wait gave up (s.error is then set).
__device__ __forceinline__ bool tc_forward(TcSmem &s, uint32_t &phase, float *o)
{
    bool ok = tc_layer(s, s.x, kMlpInPad, s.w1, kMlpHid, phase);
    tc_hidden_epilogue(s, s.b1);
    ok = tc_layer(s, s.h, kMlpHid, s.w2, kMlpHid, phase) && ok;
    tc_hidden_epilogue(s, s.b2);
    ok = tc_layer(s, s.h, kMlpHid, s.w3, kMlpOutPad, phase) && ok;
    const uint32_t lane_base = s.tmem + ((uint32_t)(threadIdx.x & ~31) << 16);
    float v[16];
    tmem_ld16(lane_base, v);
#pragma unroll
    for (int i = 0; i < 16; ++i) o[i] = v[i] + s.b3[i];
    tmem_ld16(lane_base + 16u, v);
#pragma unroll
    for (int i = 0; i < kMlpOut - 16; ++i) o[16 + i] = v[i] + s.b3[16 + i];
    // the next layer 1 overwrites the accumulators: every load done first
    tc_fence_before();
    return ok;
}

}  // namespace esp
