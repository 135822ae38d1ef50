// Training GEMMs of the learned proposal on the tcgen05 tensor cores:
// C[M][N] = op(A) op(B) with BF16 operands and FP32 accumulation in tensor
// memory, for the forward pass (M = batch, N = 128 or 32, K = 16 or 128),
// the input gradients (M = batch) and the weight gradients (M, N <= 128,
// K = batch, split over CTAs along K into a workspace of partial tiles that a
// second kernel adds in a fixed order, so results do not depend on timing).
//
// A CTA of 128 threads owns one 128-row tile of C and up to 128 columns:
// thread t stages operand chunks into shared memory, and owns row t of the
// tile (its tensor-memory lane) in the epilogue.  Both operands sit in shared
// memory in the K-major no-swizzle layout of esp_tc.cuh whatever their order
// in global memory: the staging copy transposes the operands stored [K][M]
// (TA) or [K][N] (TB), so every MMA is the K-major form that the learned
// sweep's network also uses.  Per K-chunk of 64, one thread issues four
// tcgen05.mma (K = 16 each) and commits them to an mbarrier that every thread
// waits on with an iteration limit; a wait that gives up sets *err, and the
// CTA then stops issuing, writes nothing, waits once more (bounded) for the
// MMAs in flight and frees its tensor memory.
#include <cuda_bf16.h>

#include "esp_learned.h"
#include "esp_lp_tc.cuh"
#include "esp_tc.cuh"

namespace esp {

namespace {

constexpr int kGtM = 128;        // rows of a tile (tensor-memory lanes)
constexpr int kGtK = 64;         // K-chunk staged per round
constexpr int kGtThreads = 128;

struct alignas(128) GemmTcSmem {
    __nv_bfloat16 a[kGtM * kGtK];       // [128][64] K-major
    __nv_bfloat16 b[kGtM * kGtK];       // [<=128][64] K-major
    unsigned long long bar;
    uint32_t tmem;
};

// Dynamic shared memory per CTA: more than the operands need, so that at most
// three CTAs share an SM and their tensor-memory allocations (up to 128
// columns each) fit the SM's 512 columns without waiting.
constexpr size_t kGemmTcSmemBytes = 72 * 1024;

// Tensor-memory columns to allocate for n accumulator columns (a power of
// two, at least 32).
__host__ __device__ constexpr uint32_t tmem_cols_for(int n) { return n <= 32 ? 32u : (n <= 64 ? 64u : 128u); }

template <bool TA, bool TB>
__global__ void __launch_bounds__(kGtThreads) k_gemm_tc(const GemmArgs g, int BN, int k_per_cta, float *part, int *err)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    GemmTcSmem &s = *reinterpret_cast<GemmTcSmem *>(smem_raw);
    const int t = threadIdx.x;
    const int m0 = blockIdx.x * kGtM, n0 = blockIdx.y * BN;
    const int kb = blockIdx.z * k_per_cta, ke = min(g.K, kb + k_per_cta);
    const uint32_t ncols = tmem_cols_for(BN);
    if (t == 0) mbar_init(smem_u32(&s.bar), 1);
    if (t < 32) {
        tmem_alloc(smem_u32(&s.tmem), ncols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t idesc = idesc_bf16_f32(kGtM, BN);
    uint32_t phase = 0;
    bool ok = true, pending = false;
    unsigned char *ab = reinterpret_cast<unsigned char *>(s.a);
    unsigned char *bb = reinterpret_cast<unsigned char *>(s.b);
    for (int k0 = kb; k0 < ke; k0 += kGtK) {
        // ---- stage A rows m0..m0+127 and B rows n0..n0+BN-1, columns k0..k0+63
        for (int ch = t; ch < kGtM * (kGtK / 8); ch += kGtThreads) {
            if (!TA) {   // A stored [M][K]: 8 consecutive k of one row
                const int r = ch / (kGtK / 8), kc = (ch % (kGtK / 8)) * 8;
                const int gm = m0 + r, gk = k0 + kc;
                uint4 v = make_uint4(0u, 0u, 0u, 0u);
                if (gm < g.M && gk < ke) v = *reinterpret_cast<const uint4 *>(g.A + (size_t)gm * g.lda + gk);
                *reinterpret_cast<uint4 *>(ab + kmajor_offset(r, kc, kGtK)) = v;
            } else {     // A stored [K][M]: 8 consecutive m of one k, scattered into 8 rows
                const int kk = ch / (kGtM / 8), rc = (ch % (kGtM / 8)) * 8;
                const int gk = k0 + kk, gm = m0 + rc;
                uint4 v = make_uint4(0u, 0u, 0u, 0u);
                if (gk < ke && gm < g.M) v = *reinterpret_cast<const uint4 *>(g.A + (size_t)gk * g.lda + gm);
                const __nv_bfloat16 *e = reinterpret_cast<const __nv_bfloat16 *>(&v);
#pragma unroll
                for (int i = 0; i < 8; ++i)
                    *reinterpret_cast<__nv_bfloat16 *>(ab + kmajor_offset(rc + i, kk, kGtK)) = e[i];
            }
        }
        for (int ch = t; ch < BN * (kGtK / 8); ch += kGtThreads) {
            if (!TB) {   // B stored [N][K]
                const int r = ch / (kGtK / 8), kc = (ch % (kGtK / 8)) * 8;
                const int gn = n0 + r, gk = k0 + kc;
                uint4 v = make_uint4(0u, 0u, 0u, 0u);
                if (gn < g.N && gk < ke) v = *reinterpret_cast<const uint4 *>(g.B + (size_t)gn * g.ldb + gk);
                *reinterpret_cast<uint4 *>(bb + kmajor_offset(r, kc, kGtK)) = v;
            } else {     // B stored [K][N]
                const int nb = BN / 8;
                const int kk = ch / nb, rc = (ch % nb) * 8;
                const int gk = k0 + kk, gn = n0 + rc;
                uint4 v = make_uint4(0u, 0u, 0u, 0u);
                if (gk < ke && gn < g.N) v = *reinterpret_cast<const uint4 *>(g.B + (size_t)gk * g.ldb + gn);
                const __nv_bfloat16 *e = reinterpret_cast<const __nv_bfloat16 *>(&v);
#pragma unroll
                for (int i = 0; i < 8; ++i)
                    *reinterpret_cast<__nv_bfloat16 *>(bb + kmajor_offset(rc + i, kk, kGtK)) = e[i];
            }
        }
        // ---- the staged operands -> tensor cores; one thread issues
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (t == 0) {
            const uint32_t sbo = (uint32_t)(kGtK / 8) * 128u;
            const uint32_t a0 = smem_u32(s.a), b0 = smem_u32(s.b);
#pragma unroll
            for (int kk = 0; kk < kGtK / 16; ++kk)
                tc_mma(s.tmem, smem_desc(a0 + 256u * kk, 128u, sbo), smem_desc(b0 + 256u * kk, 128u, sbo), idesc,
                       (k0 > kb || kk > 0) ? 1u : 0u);
            tc_commit(smem_u32(&s.bar));
        }
        const bool seen = mbar_wait(smem_u32(&s.bar), phase, kTcWaitLimit);
        // the same decision for every thread of the CTA
        const bool fail = __syncthreads_or(!seen) != 0;
        if (fail) {
            pending = __syncthreads_or(seen) == 0;
            if (!pending) phase ^= 1u;
            ok = false;
            break;
        }
        phase ^= 1u;
        tc_fence_after();
    }
    if (ok && kb < ke) {
        // ---- epilogue: row t of the tile, 16 columns per tensor-memory load
        const int m = m0 + t;
        const uint32_t lane_base = s.tmem + ((uint32_t)(t & ~31) << 16);
        for (int c0 = 0; c0 < BN; c0 += 16) {
            float v[16];
            tmem_ld16(lane_base + (uint32_t)c0, v);
            if (m >= g.M) continue;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int n = n0 + c0 + j;
                if (n >= g.N) continue;
                float x = v[j];
                if (g.bias) x += g.bias[n];
                if (g.relu) x = fmaxf(x, 0.f);
                if (g.mask && !(__bfloat162float(g.mask[(size_t)m * g.ldm + n]) > 0.f)) x = 0.f;
                if (part) {   // split K: this CTA's partial, [split][M][N]
                    part[((size_t)blockIdx.z * g.M + m) * g.N + n] = x;
                } else if (g.C) {
                    float *o = g.C + (size_t)m * g.ldc + n;
                    *o = g.accumulate ? *o + x : x;
                }
                if (g.Cb) g.Cb[(size_t)m * g.ldcb + n] = __float2bfloat16_rn(x);
            }
        }
    }
    if (!ok && t == 0) atomicExch(err, 1);
    // a give-up with MMAs possibly still running: wait for them once more
    // (bounded) before the tensor memory is freed
    if (pending && t == 0) mbar_wait(smem_u32(&s.bar), phase, kTcWaitLimit);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (t < 32) tmem_dealloc(s.tmem, ncols);
}

// C[m][n] = sum over the splits in order of part[z][m][n]
__global__ void k_gemm_tc_reduce(const float *part, int splits, int M, int N, float *C, int ldc)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M * N) return;
    float acc = 0.f;
    for (int z = 0; z < splits; ++z) acc += part[(size_t)z * M * N + i];
    C[(size_t)(i / N) * ldc + i % N] = acc;
}

int split_count(const GemmArgs &g, int num_sms, int &k_per)
{
    const int BN = g.N <= 128 ? g.N : 128;
    const int mt = (g.M + kGtM - 1) / kGtM, nt = (g.N + BN - 1) / BN;
    int splits = 1;
    if (g.C && !g.Cb && !g.bias && !g.relu && !g.mask && !g.accumulate && g.M * g.N <= kGemmTcSplitMN) {
        const int want = (2 * num_sms) / (mt * nt);
        const int max_split = (g.K + kGtK - 1) / kGtK;
        splits = want < 1 ? 1 : (want > max_split ? max_split : want);
        if (splits > kGemmTcMaxSplit) splits = kGemmTcMaxSplit;
    }
    k_per = (g.K + splits - 1) / splits;
    k_per = (k_per + kGtK - 1) / kGtK * kGtK;
    return (g.K + k_per - 1) / k_per;
}

}  // namespace

cudaError_t gemm_tc_configure()
{
    static_assert(sizeof(GemmTcSmem) <= kGemmTcSmemBytes, "operand tiles exceed the shared-memory request");
    const int bytes = (int)kGemmTcSmemBytes;
    cudaError_t e = cudaFuncSetAttribute(k_gemm_tc<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_gemm_tc<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_gemm_tc<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_gemm_tc<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    return e;
}

cudaError_t launch_gemm_tc(const GemmArgs &g, bool ta, bool tb, int num_sms, float *work, int *err, cudaStream_t st)
{
    // 16-byte staging loads and the MMA shape: N a multiple of 16, the
    // leading dimensions multiples of 8, at most 128 columns per tile
    if (g.M <= 0 || g.N <= 0 || g.K <= 0 || (g.M & 7) || (g.K & 7) || (g.lda & 7) || (g.ldb & 7) || (g.N & 15) ||
        (reinterpret_cast<uintptr_t>(g.A) & 15) || (reinterpret_cast<uintptr_t>(g.B) & 15))
        return cudaErrorInvalidValue;
    const int BN = g.N <= 128 ? g.N : 128;
    const int mt = (g.M + kGtM - 1) / kGtM, nt = (g.N + BN - 1) / BN;
    // weight gradients (few tiles, long K): split K over CTAs, each writing a
    // partial tile to the workspace, then a fixed-order sum into C
    int k_per = 0;
    const int splits = split_count(g, num_sms, k_per);
    if (splits > 1 && !work) return cudaErrorInvalidValue;
    float *part = splits > 1 ? work : nullptr;
    const dim3 grid(mt, nt, splits);
    const size_t sm = kGemmTcSmemBytes;
    if (!ta && !tb) k_gemm_tc<false, false><<<grid, kGtThreads, sm, st>>>(g, BN, k_per, part, err);
    else if (ta && tb) k_gemm_tc<true, true><<<grid, kGtThreads, sm, st>>>(g, BN, k_per, part, err);
    else if (!ta) k_gemm_tc<false, true><<<grid, kGtThreads, sm, st>>>(g, BN, k_per, part, err);
    else k_gemm_tc<true, false><<<grid, kGtThreads, sm, st>>>(g, BN, k_per, part, err);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && part) {
        k_gemm_tc_reduce<<<(g.M * g.N + 255) / 256, 256, 0, st>>>(part, splits, g.M, g.N, g.C, g.ldc);
        e = cudaGetLastError();
    }
    return e;
}

}  // namespace esp
