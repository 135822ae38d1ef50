// BF16 tensor-core building blocks of the learned proposal's MLP
// (12 -> 128 -> 128 -> 20, ReLU, FP32 accumulation), warp-level
// mma.m16n8k16 with ldmatrix fragment loads.
//
// Weights are kept as [out][in] rows (in contiguous), which is the "col"
// operand layout of mma.m16n8k16.  In shared memory every row is padded by 8
// elements so that the 8 rows one ldmatrix reads fall in distinct banks.
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

#include "esp_vmf.cuh"

namespace esp {

constexpr int kLdw1 = kMlpInPad + 8;   // padded row lengths (bf16 elements)
constexpr int kLdw2 = kMlpHid + 8;
constexpr int kLdx = kMlpInPad + 8;
constexpr int kLdh = kMlpHid + 8;
constexpr int kLdo = kMlpOutPad + 1;   // floats

// Device copies of the network (padded): W1 [128][16], W2 [128][128],
// W3 [32][128] in bf16; biases b1 [128], b2 [128], b3 [32] in fp32.
struct LpWeights {
    const __nv_bfloat16 *w1, *w2, *w3;
    const float *b1, *b2, *b3;
};

__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void ldsm_x4(uint32_t r[4], const __nv_bfloat16 *p)
{
    const unsigned addr = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(addr));
}

__device__ __forceinline__ void ldsm_x4_t(uint32_t r[4], const __nv_bfloat16 *p)
{
    const unsigned addr = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(addr));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&v);
}

// Fragment addresses (lane l, j = l >> 3, i = l & 7) for x4 loads:
//  A from [m][k] storage: row m0 + (l & 15), column k0 + (l >> 4) * 8
//    -> a0..a3 of m16n8k16;
//  B from [n][k] storage: row n0 + i + (j >> 1) * 8, column k0 + (j & 1) * 8
//    -> {r0, r1} = B fragment of n-tile n0, {r2, r3} of n-tile n0 + 8.
__device__ __forceinline__ const __nv_bfloat16 *a_addr(const __nv_bfloat16 *base, int ld, int m0, int k0, int lane)
{
    return base + (m0 + (lane & 15)) * ld + k0 + ((lane >> 4) << 3);
}
__device__ __forceinline__ const __nv_bfloat16 *b_addr(const __nv_bfloat16 *base, int ld, int n0, int k0, int lane)
{
    return base + (n0 + (lane & 7) + ((lane >> 4) << 3)) * ld + k0 + (((lane >> 3) & 1) << 3);
}

// Shared-memory copy of the weights (padded rows) and biases.
struct LpSmemWeights {
    __nv_bfloat16 w1[kMlpHid * kLdw1];
    __nv_bfloat16 w2[kMlpHid * kLdw2];
    __nv_bfloat16 w3[kMlpOutPad * kLdw2];
    float b1[kMlpHid], b2[kMlpHid], b3[kMlpOutPad];
};

__device__ __forceinline__ void lp_stage_weights(const LpWeights &w, LpSmemWeights &s)
{
    // 16-byte chunks: 2 per W1 row, 16 per W2/W3 row
    for (int i = threadIdx.x; i < kMlpHid * 2; i += blockDim.x)
        *reinterpret_cast<uint4 *>(s.w1 + (i >> 1) * kLdw1 + (i & 1) * 8) =
            __ldg(reinterpret_cast<const uint4 *>(w.w1) + i);
    for (int i = threadIdx.x; i < kMlpHid * 16; i += blockDim.x)
        *reinterpret_cast<uint4 *>(s.w2 + (i >> 4) * kLdw2 + (i & 15) * 8) =
            __ldg(reinterpret_cast<const uint4 *>(w.w2) + i);
    for (int i = threadIdx.x; i < kMlpOutPad * 16; i += blockDim.x)
        *reinterpret_cast<uint4 *>(s.w3 + (i >> 4) * kLdw2 + (i & 15) * 8) =
            __ldg(reinterpret_cast<const uint4 *>(w.w3) + i);
    for (int i = threadIdx.x; i < kMlpHid; i += blockDim.x) { s.b1[i] = __ldg(w.b1 + i); s.b2[i] = __ldg(w.b2 + i); }
    for (int i = threadIdx.x; i < kMlpOutPad; i += blockDim.x) s.b3[i] = __ldg(w.b3 + i);
}

// Per-warp scratch: inputs X [32][kLdx] and activations H [32][kLdh] (bf16);
// layer 2 runs in place on H and the FP32 outputs [32][kLdo] overlay H.
struct LpWarpBuf {
    __nv_bfloat16 x[32 * kLdx];
    __nv_bfloat16 h[32 * kLdh];
};
static_assert(32 * kLdo * sizeof(float) <= sizeof(__nv_bfloat16) * 32 * kLdh, "outputs must fit over H");

__device__ __forceinline__ float *lp_out_rows(LpWarpBuf &b) { return reinterpret_cast<float *>(b.h); }

// One hidden layer with K = 128 in place on H: H <- relu(H W^T + bias).
__device__ __forceinline__ void lp_hidden128(const __nv_bfloat16 *w, const float *bias, __nv_bfloat16 *h, int lane)
{
    uint32_t a[2][8][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int kt = 0; kt < 8; ++kt) ldsm_x4(a[mt][kt], a_addr(h, kLdh, mt * 16, kt * 16, lane));
    __syncwarp();
    const int g = lane >> 2, t = lane & 3;
#pragma unroll 1
    for (int np = 0; np < kMlpHid / 16; ++np) {
        float c[2][2][4] = {};
#pragma unroll
        for (int kt = 0; kt < 8; ++kt) {
            uint32_t b[4];
            ldsm_x4(b, b_addr(w, kLdw2, np * 16, kt * 16, lane));
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                mma_bf16(c[mt][0], a[mt][kt], b[0], b[1]);
                mma_bf16(c[mt][1], a[mt][kt], b[2], b[3]);
            }
        }
#pragma unroll
        for (int nt = 0; nt < 2; ++nt) {
            const int col = np * 16 + nt * 8 + 2 * t;
            const float b0 = bias[col], b1 = bias[col + 1];
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                *reinterpret_cast<uint32_t *>(h + (mt * 16 + g) * kLdh + col) =
                    pack_bf16(fmaxf(c[mt][nt][0] + b0, 0.f), fmaxf(c[mt][nt][1] + b1, 0.f));
                *reinterpret_cast<uint32_t *>(h + (mt * 16 + g + 8) * kLdh + col) =
                    pack_bf16(fmaxf(c[mt][nt][2] + b0, 0.f), fmaxf(c[mt][nt][3] + b1, 0.f));
            }
        }
    }
    __syncwarp();
}

// Forward pass of 32 samples (rows of b.x, one per lane): FP32 outputs in
// lp_out_rows(b), row stride kLdo, the first kMlpOut columns used.  Every
// lane of the warp must call it.
__device__ __forceinline__ void lp_warp_forward(const LpSmemWeights &w, LpWarpBuf &b)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    // layer 1: [32 x 16] . [16 x 128]
    {
        uint32_t a[2][4];
        ldsm_x4(a[0], a_addr(b.x, kLdx, 0, 0, lane));
        ldsm_x4(a[1], a_addr(b.x, kLdx, 16, 0, lane));
#pragma unroll 2
        for (int np = 0; np < kMlpHid / 16; ++np) {
            uint32_t bb[4];
            ldsm_x4(bb, b_addr(w.w1, kLdw1, np * 16, 0, lane));
#pragma unroll
            for (int nt = 0; nt < 2; ++nt) {
                const int col = np * 16 + nt * 8 + 2 * t;
                const float b0 = w.b1[col], b1 = w.b1[col + 1];
#pragma unroll
                for (int mt = 0; mt < 2; ++mt) {
                    float c[4] = {0.f, 0.f, 0.f, 0.f};
                    mma_bf16(c, a[mt], bb[2 * nt], bb[2 * nt + 1]);
                    *reinterpret_cast<uint32_t *>(b.h + (mt * 16 + g) * kLdh + col) =
                        pack_bf16(fmaxf(c[0] + b0, 0.f), fmaxf(c[1] + b1, 0.f));
                    *reinterpret_cast<uint32_t *>(b.h + (mt * 16 + g + 8) * kLdh + col) =
                        pack_bf16(fmaxf(c[2] + b0, 0.f), fmaxf(c[3] + b1, 0.f));
                }
            }
        }
    }
    __syncwarp();
    // layer 2: [32 x 128] . [128 x 128], in place
    lp_hidden128(w.w2, w.b2, b.h, lane);
    // layer 3: [32 x 128] . [128 x 32] -> FP32 rows over H
    {
        uint32_t a[2][8][4];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
            for (int kt = 0; kt < 8; ++kt) ldsm_x4(a[mt][kt], a_addr(b.h, kLdh, mt * 16, kt * 16, lane));
        __syncwarp();
        float *out = lp_out_rows(b);
#pragma unroll 1
        for (int np = 0; np < kMlpOutPad / 16; ++np) {
            float c[2][2][4] = {};
#pragma unroll
            for (int kt = 0; kt < 8; ++kt) {
                uint32_t bb[4];
                ldsm_x4(bb, b_addr(w.w3, kLdw2, np * 16, kt * 16, lane));
#pragma unroll
                for (int mt = 0; mt < 2; ++mt) {
                    mma_bf16(c[mt][0], a[mt][kt], bb[0], bb[1]);
                    mma_bf16(c[mt][1], a[mt][kt], bb[2], bb[3]);
                }
            }
#pragma unroll
            for (int nt = 0; nt < 2; ++nt) {
                const int col = np * 16 + nt * 8 + 2 * t;
                const float b0 = w.b3[col], b1 = w.b3[col + 1];
#pragma unroll
                for (int mt = 0; mt < 2; ++mt) {
                    out[(mt * 16 + g) * kLdo + col] = c[mt][nt][0] + b0;
                    out[(mt * 16 + g) * kLdo + col + 1] = c[mt][nt][1] + b1;
                    out[(mt * 16 + g + 8) * kLdo + col] = c[mt][nt][2] + b0;
                    out[(mt * 16 + g + 8) * kLdo + col + 1] = c[mt][nt][3] + b1;
                }
            }
        }
    }
    __syncwarp();
}

}  // namespace esp
