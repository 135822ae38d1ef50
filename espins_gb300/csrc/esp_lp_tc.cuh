// The learned proposal's MLP (12 -> 128 -> 128 -> 20, ReLU) on the tcgen05
// tensor cores for tiles of 128 rows: a group of 128 threads (a warpgroup)
// owns one tile, thread t of the group owns row t (its tensor-memory lane).
// A CTA holds NG groups that share one copy of the weights and work on their
// tiles independently (named barrier 1 + g per group); group g accumulates in
// tensor-memory columns [128 g, 128 g + 128).  Operands in shared memory in
// the K-major no-swizzle layout of esp_tc.cuh, one thread per group issues
// the MMAs and an mbarrier per group signals their completion.
#pragma once
#include <cuda_bf16.h>

#include "esp_mlp.cuh"
#include "esp_tc.cuh"

namespace esp {

constexpr int kTcRows = 128;
constexpr uint32_t kTcCols = 128;           // tensor-memory columns per group
constexpr int kTcGroups = 4;                // groups (tiles in flight) per CTA of the sweep
constexpr uint32_t kTcWaitLimit = 1u << 24; // mbarrier polls before giving up

// One group's tile: features X, hidden activations H, completion barrier.
struct alignas(128) TcTile {
    __nv_bfloat16 x[kTcRows * kMlpInPad];      // [128][16]
    __nv_bfloat16 h[kTcRows * kMlpHid];        // [128][128]
    unsigned long long bar;
};

template <int NG>
struct TcSmemG {
    __nv_bfloat16 w1[kMlpHid * kMlpInPad];     // [128][16] K-major
    __nv_bfloat16 w2[kMlpHid * kMlpHid];       // [128][128]
    __nv_bfloat16 w3[kMlpOutPad * kMlpHid];    // [32][128]
    float b1[kMlpHid], b2[kMlpHid], b3[kMlpOutPad];
    TcTile t[NG];
    uint32_t tmem;
    int error;
};
using TcSmem = TcSmemG<1>;

// Barrier of group g's 128 threads (the whole CTA when there is one group).
template <int NG>
__device__ __forceinline__ void group_sync(int g)
{
    if (NG == 1) __syncthreads();
    else asm volatile("bar.sync %0, 128;\n" ::"r"(g + 1) : "memory");
}

// OR of v over group g's 128 threads, with that group's barrier.
template <int NG>
__device__ __forceinline__ bool group_any(int g, bool v)
{
    if (NG == 1) return __syncthreads_or(v) != 0;
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.or.pred q, %2, 128, p;\n\tselp.u32 %0, 1, 0, q;\n\t}\n"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(g + 1)
        : "memory");
    return r != 0;
}

// Row-major global weights ([out][in]) to the K-major operand layout.
template <int NG>
__device__ __forceinline__ void tc_stage_weights(const LpWeights &w, TcSmemG<NG> &s)
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

// Set-up by the whole CTA: one mbarrier per group, 128 tensor-memory columns
// per group (warp 0).
template <int NG>
__device__ __forceinline__ void tc_setup(TcSmemG<NG> &s)
{
    if (threadIdx.x == 0) {
        for (int g = 0; g < NG; ++g) mbar_init(smem_u32(&s.t[g].bar), 1);
        s.error = 0;
    }
    if (threadIdx.x < 32) {
        tmem_alloc(smem_u32(&s.tmem), kTcCols * NG);
        tmem_relinquish();
    }
    // every thread's weight writes -> the tensor cores of every group
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
}

// Tear-down by the whole CTA.  A group whose completion wait gave up with its
// MMAs possibly still in flight (pending) first waits for them once more,
// bounded, so the tensor memory is not freed under a running MMA; if that
// wait gives up too, the memory is freed regardless (the launch has already
// reported the error).
template <int NG>
__device__ __forceinline__ void tc_teardown(TcSmemG<NG> &s, int g = 0, bool pending = false, uint32_t phase = 0)
{
    if (pending && (threadIdx.x & (kTcRows - 1)) == 0) mbar_wait(smem_u32(&s.t[g].bar), phase, kTcWaitLimit);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (threadIdx.x < 32) tmem_dealloc(s.tmem, kTcCols * NG);
}

// Thread t's 12 features as row t of the X operand (zero padding to 16).
__device__ __forceinline__ void tc_store_x_row(TcTile &s, int t, const float *f)
{
    uint4 v0, v1;
    v0.x = pack_bf16(f[0], f[1]); v0.y = pack_bf16(f[2], f[3]); v0.z = pack_bf16(f[4], f[5]); v0.w = pack_bf16(f[6], f[7]);
    v1.x = pack_bf16(f[8], f[9]); v1.y = pack_bf16(f[10], f[11]); v1.z = 0u; v1.w = 0u;
    unsigned char *b = reinterpret_cast<unsigned char *>(s.x);
    *reinterpret_cast<uint4 *>(b + kmajor_offset(t, 0, kMlpInPad)) = v0;
    *reinterpret_cast<uint4 *>(b + kmajor_offset(t, 8, kMlpInPad)) = v1;
}

// Issue (the group's thread 0) the MMAs of one layer of group g, commit, and
// wait (every thread of the group).  Returns true, the same for every thread
// of the group, when the layer's results are in tensor memory.  When a wait
// gives up (or `force` asks the test hook to report a give-up after the MMAs
// completed) it returns false and sets s.error; `pending` then tells whether
// the MMAs may still be running (no thread of the group saw them complete),
// and `phase` is the phase still to wait for.  After a false return the
// group must issue no more MMAs and read neither tensor memory nor touch the
// operands the MMAs read.
template <int NG>
__device__ __forceinline__ bool tc_layer(TcSmemG<NG> &s, int g, const __nv_bfloat16 *a, int K,
                                         const __nv_bfloat16 *b, int N, uint32_t &phase, int force, bool &pending)
{
    fence_async_smem();     // this thread's operand writes -> tensor cores
    tc_fence_before();
    group_sync<NG>(g);
    tc_fence_after();
    if ((threadIdx.x & (kTcRows - 1)) == 0) {
        const uint32_t idesc = idesc_bf16_f32(kTcRows, N);
        const uint32_t sbo = (uint32_t)(K / 8) * 128u;
        const uint32_t a0 = smem_u32(a), b0 = smem_u32(b);
        const uint32_t d = s.tmem + kTcCols * (uint32_t)g;
        for (int kk = 0; kk < K / 16; ++kk)
            tc_mma(d, smem_desc(a0 + 256u * kk, 128u, sbo), smem_desc(b0 + 256u * kk, 128u, sbo), idesc, kk > 0);
        tc_commit(smem_u32(&s.t[g].bar));
    }
    const bool seen = mbar_wait(smem_u32(&s.t[g].bar), phase, kTcWaitLimit);
    const bool fail = group_any<NG>(g, !seen || force != 0);
    if (!fail) {
        phase ^= 1u;
        tc_fence_after();
        return true;
    }
    // give-up: the layer's MMAs are complete if any thread of the group saw it
    const bool done = group_any<NG>(g, seen);
    if (done) phase ^= 1u;
    pending = !done;
    if ((threadIdx.x & (kTcRows - 1)) == 0) s.error = 1;
    return false;
}

// This thread's tensor-memory lane in group g's columns.
template <int NG>
__device__ __forceinline__ uint32_t tc_lane_base(const TcSmemG<NG> &s, int g)
{
    const int t = threadIdx.x & (kTcRows - 1);
    return s.tmem + kTcCols * (uint32_t)g + ((uint32_t)(t & ~31) << 16);
}

// Hidden-layer epilogue: relu(D + bias) of this thread's row to group g's H.
template <int NG>
__device__ __forceinline__ void tc_hidden_epilogue(TcSmemG<NG> &s, int g, const float *bias)
{
    const int t = threadIdx.x & (kTcRows - 1);
    const uint32_t lane_base = tc_lane_base(s, g);
    unsigned char *hb = reinterpret_cast<unsigned char *>(s.t[g].h);
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

// The whole network for the 128 rows of group g's X; thread t of the group
// gets row t's 20 outputs.  Returns false (for the whole group) if a wait
// gave up: s.error is then set, `pending` says whether MMAs may still run, and
// neither o nor the group's operands or tensor memory have been touched
// after the failed layer.
template <int NG>
__device__ __forceinline__ bool tc_forward(TcSmemG<NG> &s, int g, uint32_t &phase, float *o, int force,
                                           bool &pending)
{
    TcTile &tl = s.t[g];
    if (!tc_layer(s, g, tl.x, kMlpInPad, s.w1, kMlpHid, phase, force, pending)) return false;
    tc_hidden_epilogue(s, g, s.b1);
    if (!tc_layer(s, g, tl.h, kMlpHid, s.w2, kMlpHid, phase, 0, pending)) return false;
    tc_hidden_epilogue(s, g, s.b2);
    if (!tc_layer(s, g, tl.h, kMlpHid, s.w3, kMlpOutPad, phase, 0, pending)) return false;
    const uint32_t lane_base = tc_lane_base(s, g);
    float v[16];
    tmem_ld16(lane_base, v);
#pragma unroll
    for (int i = 0; i < 16; ++i) o[i] = v[i] + s.b3[i];
    tmem_ld16(lane_base + 16u, v);
#pragma unroll
    for (int i = 0; i < kMlpOut - 16; ++i) o[16 + i] = v[i] + s.b3[16 + i];
    // the next layer 1 overwrites the accumulators: every load done first
    tc_fence_before();
    return true;
}

}  // namespace esp
