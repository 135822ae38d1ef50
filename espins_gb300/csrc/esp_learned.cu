// Learned proposal kernels.
//
//   k_sweep_lp       one colour class of a Metropolis-Hastings sweep whose
//                    trial spin comes from the vMF mixture an MLP predicts
//                    from the site's environment (BF16 mma.sync, FP32
//                    accumulation, weights resident in shared memory)
//   k_lp_collect     training pairs (features, spin in the local frame) from
//                    the current configurations of the plain sampler
//   k_gemm_bf16      C = op(A) op(B) for the training passes, with fused
//                    bias / ReLU / ReLU-mask epilogues
//   k_lp_head        loss -mean log q(s) and its gradient w.r.t. the outputs
//   k_colsum, k_adam, k_lp_to_bf16, k_lp_gather, k_lp_forward
//
// The spin update, its bookkeeping and the random stream follow k_sweep_ell
// (metropolis, get_quant.F90:52-182, with the acceptance test of a
// non-symmetric proposal); the network and its training have no counterpart
// in the reference.
#include "esp_learned.h"
#include "esp_lp_tc.cuh"

namespace esp {

namespace {

// Linear field g and quadratic form Q (xx, yy, zz, xy, xz, yz) of permuted
// site p in replica r: E_p(s) = g.s + s^T Q s (delta_energy_get,
// get_quant.F90:294-333, in local form).
template <bool HB, bool HD>
__device__ __forceinline__ void site_terms(const SweepArgs &a, int p, int r, int orig, float &gx, float &gy,
                                           float &gz, float q[6])
{
    const int R = a.R;
    gx = gy = gz = 0.f;
    for (int i = 0; i < 6; ++i) q[i] = 0.f;
    const int nn = __ldg(a.nnb + p);
    for (int k0 = 0; k0 < nn; k0 += 8) {
        int nb[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) nb[j] = __ldg(a.nbr + (size_t)(k0 + j) * a.N + p);
        float tx[8], ty[8], tz[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const size_t iq = (size_t)nb[j] * R + r;
            tx[j] = __ldg(a.sx + iq); ty[j] = __ldg(a.sy + iq); tz[j] = __ldg(a.sz + iq);
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const size_t e = (size_t)(k0 + j) * a.N + p;
            const float J = __ldg(a.J + e);
            gx = fmaf(-J, tx[j], gx); gy = fmaf(-J, ty[j], gy); gz = fmaf(-J, tz[j], gz);
            if (HB) {
                const float Bv = __ldg(a.B + e);
                const float bx = Bv * tx[j], by = Bv * ty[j], bz = Bv * tz[j];
                q[0] = fmaf(bx, tx[j], q[0]); q[1] = fmaf(by, ty[j], q[1]); q[2] = fmaf(bz, tz[j], q[2]);
                q[3] = fmaf(bx, ty[j], q[3]); q[4] = fmaf(bx, tz[j], q[4]); q[5] = fmaf(by, tz[j], q[5]);
            }
            if (HD) {
                const float dx = __ldg(a.Dx + e), dy = __ldg(a.Dy + e), dz = __ldg(a.Dz + e);
                gx += ty[j] * dz - tz[j] * dy;
                gy += tz[j] * dx - tx[j] * dz;
                gz += tx[j] * dy - ty[j] * dx;
            }
        }
    }
    if (a.si || a.fld) {
        const int at = orig % a.num_atoms;
        if (a.si) {
            const float4 s = __ldg(a.si + at);
            const float dx = s.w * s.x, dy = s.w * s.y, dz = s.w * s.z;
            q[0] = fmaf(dx, s.x, q[0]); q[1] = fmaf(dy, s.y, q[1]); q[2] = fmaf(dz, s.z, q[2]);
            q[3] = fmaf(dx, s.y, q[3]); q[4] = fmaf(dx, s.z, q[4]); q[5] = fmaf(dy, s.z, q[5]);
        }
        if (a.fld) {
            const float4 f = __ldg(a.fld + at);
            gx += f.x; gy += f.y; gz += f.z;
        }
    }
}

__device__ __forceinline__ void frame_axis(const float4 *axis, int orig, int num_atoms, float &ax, float &ay, float &az)
{
    ax = 1.f; ay = 0.f; az = 0.f;
    if (axis) {
        const float4 v = __ldg(axis + orig % num_atoms);
        ax = v.x; ay = v.y; az = v.z;
    }
}

__device__ __forceinline__ void store_features(__nv_bfloat16 *row, const float *f)
{
    uint4 v0, v1;
    v0.x = pack_bf16(f[0], f[1]); v0.y = pack_bf16(f[2], f[3]); v0.z = pack_bf16(f[4], f[5]); v0.w = pack_bf16(f[6], f[7]);
    v1.x = pack_bf16(f[8], f[9]); v1.y = pack_bf16(f[10], f[11]); v1.z = 0u; v1.w = 0u;
    reinterpret_cast<uint4 *>(row)[0] = v0;
    reinterpret_cast<uint4 *>(row)[1] = v1;
}

// One learned Metropolis-Hastings trial of permuted site p in replica r from
// the network outputs o: a vMF-mixture sample, both log-densities, the
// energy change of the local form g.s + s^T Q s, the test
// u < exp(-beta dE) q(old) / q(new), and the update.
__device__ __forceinline__ void lp_trial(const SweepArgs &a, const LpFrame &fr, const float *o, int p, int r, int orig,
                                         float mag, float beta, float gx, float gy, float gz, const float q[6],
                                         uint32_t sw_lo, uint32_t sw_hi, float &accE, float &accX, float &accY,
                                         float &accZ, unsigned int &nrej)
{
    VmfMix mix;
    vmf_params(o, fr.kappa0, mix);
    const size_t idx = (size_t)p * a.R + r;
    const float ox = a.sx[idx], oy = a.sy[idx], oz = a.sz[idx];
    const Philox4 x = philox4x32_10((uint32_t)orig, (uint32_t)r, sw_lo, sw_hi, a.key0, a.key1);
    float ux, uy, uz;
    vmf_sample(mix, u24f(x.x), u24f(x.y), u24f(x.z), ux, uy, uz);
    const float nx = mag * (ux * fr.e[0][0] + uy * fr.e[1][0] + uz * fr.e[2][0]);
    const float ny = mag * (ux * fr.e[0][1] + uy * fr.e[1][1] + uz * fr.e[2][1]);
    const float nz = mag * (ux * fr.e[0][2] + uy * fr.e[1][2] + uz * fr.e[2][2]);
    const float im = 1.f / mag;
    const float lx = (ox * fr.e[0][0] + oy * fr.e[0][1] + oz * fr.e[0][2]) * im;
    const float ly = (ox * fr.e[1][0] + oy * fr.e[1][1] + oz * fr.e[1][2]) * im;
    const float lz = (ox * fr.e[2][0] + oy * fr.e[2][1] + oz * fr.e[2][2]) * im;
    const float lq_new = vmf_logpdf(mix, ux, uy, uz);
    const float lq_old = vmf_logpdf(mix, lx, ly, lz);
    const float dx = nx - ox, dy = ny - oy, dz = nz - oz;
    const float px = nx + ox, py = ny + oy, pz = nz + oz;
    const float de = gx * dx + gy * dy + gz * dz
                   + dx * (q[0] * px + q[3] * py + q[4] * pz)
                   + dy * (q[3] * px + q[1] * py + q[5] * pz)
                   + dz * (q[4] * px + q[5] * py + q[2] * pz);
    // Metropolis-Hastings: accept with min(1, exp(-beta dE) q(old) / q(new))
    const float lacc = -beta * de + lq_old - lq_new;
    const bool acc = lacc >= 0.f || u24f(x.w) < expf(lacc);
    if (acc) {
        a.sx[idx] = nx; a.sy[idx] = ny; a.sz[idx] = nz;
        accE += de;
        accX += dx; accY += dy; accZ += dz;
    } else {
        ++nrej;
    }
}

constexpr int kLpThreads = 512;
constexpr int kLpWarps = kLpThreads / 32;

// Partial sums of a 512-thread block, kept as two 256-thread "virtual"
// blocks so that the slot layout (and k_fold) is the one of k_sweep_ell:
// thread t of virtual block vb works on replica (vb*256 + t) % R.
__device__ __forceinline__ void add_slots_512(float e, float mx, float my, float mz, unsigned int nrej, int R,
                                              int slots, double *part, unsigned long long *part_rej, double *s_part,
                                              unsigned int *s_rej)
{
    const int half = threadIdx.x >> 8, t = threadIdx.x & 255;
    const size_t vb = (size_t)blockIdx.x * 2 + half;
    const size_t slot = vb * slots + t;
    if (R >= 256) {
        double *o = part + 4 * slot;
        o[0] += (double)e; o[1] += (double)mx; o[2] += (double)my; o[3] += (double)mz;
        part_rej[slot] += (unsigned long long)nrej;
        return;
    }
    double *sp = s_part + 4 * (half * 256);
    unsigned int *sr = s_rej + half * 256;
    sp[4 * t] = (double)e; sp[4 * t + 1] = (double)mx; sp[4 * t + 2] = (double)my; sp[4 * t + 3] = (double)mz;
    sr[t] = nrej;
    __syncthreads();
    if (t < R) {
        double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
        unsigned long long nr = 0;
        for (int u = t; u < 256; u += R) {
            a0 += sp[4 * u]; a1 += sp[4 * u + 1]; a2 += sp[4 * u + 2]; a3 += sp[4 * u + 3];
            nr += sr[u];
        }
        double *o = part + 4 * slot;
        o[0] += a0; o[1] += a1; o[2] += a2; o[3] += a3;
        part_rej[slot] += nr;
    }
}

// ---------------------------------------------------------------------------
// Learned-proposal sweep of one colour class, all replicas.  Thread -> replica
// as in k_sweep_ell (stride a multiple of R); every warp runs the network on
// its 32 current items together, so the loop runs while any lane has work.
// ---------------------------------------------------------------------------
template <bool HB, bool HD>
__global__ void __launch_bounds__(kLpThreads, 1) k_sweep_lp(const LpSweepArgs la)
{
    extern __shared__ __align__(16) unsigned char smem[];
    LpSmemWeights &W = *reinterpret_cast<LpSmemWeights *>(smem);
    LpWarpBuf *bufs = reinterpret_cast<LpWarpBuf *>(smem + sizeof(LpSmemWeights));
    LpWarpBuf &buf = bufs[threadIdx.x >> 5];
    const SweepArgs &a = la.s;
    lp_stage_weights(la.w, W);
    __syncthreads();

    const int R = a.R;
    const int lane = threadIdx.x & 31;
    const long long nthreads = (long long)gridDim.x * blockDim.x;
    const long long S = (nthreads / R) * R;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int r = (int)(tid % R);
    const float beta = a.beta[a.temp_of[r]];
    const int pstep = (int)(S / R);
    float accE = 0.f, accX = 0.f, accY = 0.f, accZ = 0.f;
    unsigned int nrej = 0;
    uint32_t sw_lo, sw_hi;
    sweep_index(a, sw_lo, sw_hi);
    int pi = tid < S ? (int)(tid / R) : a.n_c;
    while (__any_sync(0xffffffffu, pi < a.n_c)) {
        const bool act = pi < a.n_c;
        const int p = a.off_c + (act ? pi : 0);
        const int orig = __ldg(a.perm + p);
        const float mag = __ldg(a.mag + p);
        float gx = 0.f, gy = 0.f, gz = 0.f, q[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        float f[kMlpIn];
        LpFrame fr;
        if (act) {
            site_terms<HB, HD>(a, p, r, orig, gx, gy, gz, q);
            float ax, ay, az;
            frame_axis(la.axis, orig, a.num_atoms, ax, ay, az);
            lp_frame_features(beta, mag, gx, gy, gz, q, ax, ay, az, fr, f);
        } else {
            for (int i = 0; i < kMlpIn; ++i) f[i] = 0.f;
            fr.kappa0 = 0.f;
        }
        store_features(buf.x + lane * kLdx, f);
        __syncwarp();
        lp_warp_forward(W, buf);
        float o[kMlpOut];
        {
            const float *orow = lp_out_rows(buf) + lane * kLdo;
#pragma unroll
            for (int i = 0; i < kMlpOut; ++i) o[i] = orow[i];
        }
        __syncwarp();
        if (act && mag > 0.f)
            lp_trial(a, fr, o, p, r, orig, mag, beta, gx, gy, gz, q, sw_lo, sw_hi, accE, accX, accY, accZ, nrej);
        pi += pstep;
    }
    __syncthreads();   // the warp buffers become the reduction scratch
    double *s_part = reinterpret_cast<double *>(bufs);
    unsigned int *s_rej = reinterpret_cast<unsigned int *>(s_part + 4 * kLpThreads);
    add_slots_512(accE, accX, accY, accZ, nrej, R, a.slots, a.part, a.part_rej, s_part, s_rej);
}

// ---------------------------------------------------------------------------
// The same sweep with the network on tcgen05: CTAs of kTcGroups groups of 128
// threads (one CTA per SM, the weights staged once); thread t of a group owns
// one trial and tensor-memory lane t, and each group evaluates the network on
// its 128 current trials with three chains of MMAs (K = 16, 128, 128) into its
// own 128 tensor-memory columns, independently of the other groups, so one
// group's gathers overlap another's MMAs.  Partial sums go to slots of
// 128-thread virtual blocks (thread t of virtual block b = CTA * kTcGroups +
// group works on replica (b*128 + t) % R).
// ---------------------------------------------------------------------------
template <int NG, bool HB, bool HD>
__global__ void __launch_bounds__(kTcRows * NG, 1) k_sweep_lp_tc(const LpSweepArgs la, double *part,
                                                                 unsigned long long *part_rej, int slots, int *err)
{
    extern __shared__ __align__(128) unsigned char smem[];
    TcSmemG<NG> &s = *reinterpret_cast<TcSmemG<NG> *>(smem);
    const SweepArgs &a = la.s;
    tc_stage_weights(la.w, s);
    tc_setup(s);
    const int g = threadIdx.x / kTcRows, lane = threadIdx.x % kTcRows;

    const int R = a.R;
    const long long nthreads = (long long)gridDim.x * blockDim.x;
    const long long S = (nthreads / R) * R;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int r = (int)(tid % R);
    const float beta = a.beta[a.temp_of[r]];
    const int pstep = (int)(S / R);
    float accE = 0.f, accX = 0.f, accY = 0.f, accZ = 0.f;
    unsigned int nrej = 0;
    uint32_t sw_lo, sw_hi;
    sweep_index(a, sw_lo, sw_hi);
    uint32_t phase = 0;
    bool pending = false;
    int pi = tid < S ? (int)(tid / R) : a.n_c;
    while (group_any<NG>(g, pi < a.n_c)) {
        const bool act = pi < a.n_c;
        const int p = a.off_c + (act ? pi : 0);
        const int orig = __ldg(a.perm + p);
        const float mag = __ldg(a.mag + p);
        float gx = 0.f, gy = 0.f, gz = 0.f, q[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        float f[kMlpIn];
        LpFrame fr;
        if (act) {
            site_terms<HB, HD>(a, p, r, orig, gx, gy, gz, q);
            float ax, ay, az;
            frame_axis(la.axis, orig, a.num_atoms, ax, ay, az);
            lp_frame_features(beta, mag, gx, gy, gz, q, ax, ay, az, fr, f);
        } else {
            for (int i = 0; i < kMlpIn; ++i) f[i] = 0.f;
            fr.kappa0 = 0.f;
        }
        tc_store_x_row(s.t[g], lane, f);
        float o[kMlpOut];
        // a completion wait that gave up stops the group (the same for all its
        // threads): none of its remaining trials is made, no spin written
        if (!tc_forward(s, g, phase, o, la.tc_force_timeout, pending)) break;
        if (act && mag > 0.f)
            lp_trial(a, fr, o, p, r, orig, mag, beta, gx, gy, gz, q, sw_lo, sw_hi, accE, accX, accY, accZ, nrej);
        pi += pstep;
    }
    tc_teardown(s, g, pending, phase);
    if (threadIdx.x == 0 && s.error) atomicExch(err, 1);
    // the group's activation tile becomes its reduction scratch
    __syncthreads();
    double *sp = reinterpret_cast<double *>(s.t[g].h);
    unsigned int *sr = reinterpret_cast<unsigned int *>(sp + 4 * kTcRows);
    const int t = lane;
    const size_t slot = ((size_t)blockIdx.x * NG + g) * slots + t;
    if (R >= kTcRows) {
        double *o = part + 4 * slot;
        o[0] += (double)accE; o[1] += (double)accX; o[2] += (double)accY; o[3] += (double)accZ;
        part_rej[slot] += (unsigned long long)nrej;
        return;
    }
    sp[4 * t] = (double)accE; sp[4 * t + 1] = (double)accX; sp[4 * t + 2] = (double)accY; sp[4 * t + 3] = (double)accZ;
    sr[t] = nrej;
    group_sync<NG>(g);
    if (t < R) {
        double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
        unsigned long long nr = 0;
        for (int u = t; u < kTcRows; u += R) {
            a0 += sp[4 * u]; a1 += sp[4 * u + 1]; a2 += sp[4 * u + 2]; a3 += sp[4 * u + 3];
            nr += sr[u];
        }
        double *o = part + 4 * slot;
        o[0] += a0; o[1] += a1; o[2] += a2; o[3] += a3;
        part_rej[slot] += nr;
    }
}

// Training pairs of one colour class: item i = pi * R + r for i in [0, count).
template <bool HB, bool HD>
__global__ void __launch_bounds__(256) k_lp_collect(const LpCollectArgs c)
{
    const SweepArgs &a = c.s;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < c.count; i += stride) {
        const int pi = (int)(i / a.R), r = (int)(i % a.R);
        const int p = a.off_c + pi;
        const int orig = __ldg(a.perm + p);
        const float mag = __ldg(a.mag + p);
        const float beta = a.beta[a.temp_of[r]];
        float gx, gy, gz, q[6];
        site_terms<HB, HD>(a, p, r, orig, gx, gy, gz, q);
        float ax, ay, az, f[kMlpIn];
        LpFrame fr;
        frame_axis(c.axis, orig, a.num_atoms, ax, ay, az);
        lp_frame_features(beta, mag, gx, gy, gz, q, ax, ay, az, fr, f);
        const size_t row = (size_t)(c.first + i);
        store_features(c.x + row * kMlpInPad, f);
        const size_t idx = (size_t)p * a.R + r;
        const float ox = a.sx[idx], oy = a.sy[idx], oz = a.sz[idx];
        float lx = ox * fr.e[0][0] + oy * fr.e[0][1] + oz * fr.e[0][2];
        float ly = ox * fr.e[1][0] + oy * fr.e[1][1] + oz * fr.e[1][2];
        float lz = ox * fr.e[2][0] + oy * fr.e[2][1] + oz * fr.e[2][2];
        const float n = sqrtf(lx * lx + ly * ly + lz * lz);
        const float in = n > 0.f ? 1.f / n : 0.f;
        float4 t;
        t.x = lx * in; t.y = ly * in; t.z = lz * in; t.w = fr.kappa0;
        reinterpret_cast<float4 *>(c.t)[row] = t;
    }
}

// ---------------------------------------------------------------------------
// C[M][N] = op(A) op(B), BF16 operands, FP32 accumulation.  64x64 tiles,
// k-steps of 32, four warps of 32x32.  Operands are staged in shared memory
// in their storage order (zero outside the matrix) and fragments are read
// with ldmatrix (.trans for the transposed storage orders).  Requires M, N,
// K, lda, ldb multiples of 8 and 16-byte aligned bases (checked by the
// launcher).
// ---------------------------------------------------------------------------
constexpr int kGm = 64, kGn = 64, kGk = 32;
constexpr int kGpad = 8;

template <bool TA, bool TB>
__global__ void __launch_bounds__(128) k_gemm_bf16(const GemmArgs g)
{
    // A: [kGm][kGk+pad] (TA: [kGk][kGm+pad]); B: [kGn][kGk+pad] (TB: [kGk][kGn+pad])
    constexpr int ASZ = TA ? kGk * (kGm + kGpad) : kGm * (kGk + kGpad);
    constexpr int BSZ = TB ? kGk * (kGn + kGpad) : kGn * (kGk + kGpad);
    constexpr int LDA_S = TA ? kGm + kGpad : kGk + kGpad;
    constexpr int LDB_S = TB ? kGn + kGpad : kGk + kGpad;
    __shared__ __align__(16) __nv_bfloat16 As[ASZ];
    __shared__ __align__(16) __nv_bfloat16 Bs[BSZ];
    const int m0 = blockIdx.y * kGm, n0 = blockIdx.x * kGn;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const int gq = lane >> 2, tq = lane & 3;
    float c[2][4][4] = {};
    for (int k0 = 0; k0 < g.K; k0 += kGk) {
        // 256 chunks of 8 elements per operand tile, two per thread
        for (int ch = threadIdx.x; ch < 256; ch += 128) {
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            int row, col;
            if (!TA) {
                row = ch >> 2; col = (ch & 3) * 8;
                const int gm = m0 + row, gk = k0 + col;
                if (gm < g.M && gk < g.K) v = *reinterpret_cast<const uint4 *>(g.A + (size_t)gm * g.lda + gk);
            } else {
                row = ch >> 3; col = (ch & 7) * 8;
                const int gk = k0 + row, gm = m0 + col;
                if (gk < g.K && gm < g.M) v = *reinterpret_cast<const uint4 *>(g.A + (size_t)gk * g.lda + gm);
            }
            *reinterpret_cast<uint4 *>(As + row * LDA_S + col) = v;
            v = make_uint4(0u, 0u, 0u, 0u);
            if (!TB) {
                row = ch >> 2; col = (ch & 3) * 8;
                const int gn = n0 + row, gk = k0 + col;
                if (gn < g.N && gk < g.K) v = *reinterpret_cast<const uint4 *>(g.B + (size_t)gn * g.ldb + gk);
            } else {
                row = ch >> 3; col = (ch & 7) * 8;
                const int gk = k0 + row, gn = n0 + col;
                if (gk < g.K && gn < g.N) v = *reinterpret_cast<const uint4 *>(g.B + (size_t)gk * g.ldb + gn);
            }
            *reinterpret_cast<uint4 *>(Bs + row * LDB_S + col) = v;
        }
        __syncthreads();
        const int li = lane & 7, lj = lane >> 3;
#pragma unroll
        for (int kk = 0; kk < kGk; kk += 16) {
            uint32_t af[2][4], bf[2][4];
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                if (!TA) ldsm_x4(af[mt], As + (wm + mt * 16 + (lane & 15)) * LDA_S + kk + ((lane >> 4) << 3));
                else ldsm_x4_t(af[mt], As + (kk + li + ((lj >> 1) << 3)) * LDA_S + wm + mt * 16 + ((lj & 1) << 3));
            }
#pragma unroll
            for (int np = 0; np < 2; ++np) {
                if (!TB) ldsm_x4(bf[np], Bs + (wn + np * 16 + li + ((lj >> 1) << 3)) * LDB_S + kk + ((lj & 1) << 3));
                else ldsm_x4_t(bf[np], Bs + (kk + li + ((lj & 1) << 3)) * LDB_S + wn + np * 16 + ((lj >> 1) << 3));
            }
#pragma unroll
            for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                for (int nt = 0; nt < 4; ++nt)
                    mma_bf16(c[mt][nt], af[mt], bf[nt >> 1][(nt & 1) * 2], bf[nt >> 1][(nt & 1) * 2 + 1]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
                const int m = m0 + wm + mt * 16 + gq + hh * 8;
                if (m >= g.M) continue;
#pragma unroll
                for (int cc = 0; cc < 2; ++cc) {
                    const int n = n0 + wn + nt * 8 + 2 * tq + cc;
                    if (n >= g.N) continue;
                    float v = c[mt][nt][hh * 2 + cc];
                    if (g.bias) v += g.bias[n];
                    if (g.relu) v = fmaxf(v, 0.f);
                    if (g.mask && !(__bfloat162float(g.mask[(size_t)m * g.ldm + n]) > 0.f)) v = 0.f;
                    if (g.C) {
                        float *cp = g.C + (size_t)m * g.ldc + n;
                        *cp = g.accumulate ? *cp + v : v;
                    }
                    if (g.Cb) g.Cb[(size_t)m * g.ldcb + n] = __float2bfloat16_rn(v);
                }
            }
}

// Random mini-batch (with replacement) of the training set.
__global__ void k_lp_gather(const __nv_bfloat16 *x_all, const float *t_all, long long n_all, int batch,
                            uint32_t k0, uint32_t k1, uint32_t s_lo, uint32_t s_hi, __nv_bfloat16 *xb, float *tb)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= batch) return;
    const Philox4 x = philox4x32_10((uint32_t)i, s_lo, s_hi, 0x7EA1u, k0, k1);
    const unsigned long long u = ((unsigned long long)x.x << 32) | x.y;
    // j = floor(u * n / 2^64), the high half of the 128-bit product
    const long long j = (long long)(__umul64hi(u, (unsigned long long)n_all));
    const uint4 *src = reinterpret_cast<const uint4 *>(x_all + (size_t)j * kMlpInPad);
    uint4 *dst = reinterpret_cast<uint4 *>(xb + (size_t)i * kMlpInPad);
    dst[0] = src[0]; dst[1] = src[1];
    reinterpret_cast<float4 *>(tb)[i] = reinterpret_cast<const float4 *>(t_all)[j];
}

// Loss sum_i -scale * log q(s_i) over the first n_real rows and
// d(loss)/d(outputs) in bf16 ([n_rows][32]; columns >= 20 and rows >= n_real
// zero).  One block; the loss reduction has a fixed order.
__global__ void __launch_bounds__(1024) k_lp_head(const float *o, const float *t, int n_real, int n_rows, float scale,
                                                  __nv_bfloat16 *d_o, double *loss)
{
    __shared__ double s_l[1024];
    double acc = 0.0;
    for (int i = threadIdx.x; i < n_rows; i += blockDim.x) {
        float d[kMlpOut];
        for (int k = 0; k < kMlpOut; ++k) d[k] = 0.f;
        if (i < n_real) {
            const float4 tv = reinterpret_cast<const float4 *>(t)[i];
            VmfMix mix;
            vmf_params(o + (size_t)i * kMlpOutPad, tv.w, mix);
            const float lq = vmf_logpdf_grad(mix, tv.x, tv.y, tv.z, d);
            acc += -(double)lq;
        }
        __nv_bfloat16 *row = d_o + (size_t)i * kMlpOutPad;
        for (int k = 0; k < kMlpOut; ++k) row[k] = __float2bfloat16_rn(-scale * d[k]);
        for (int k = kMlpOut; k < kMlpOutPad; ++k) row[k] = __float2bfloat16_rn(0.f);
    }
    s_l[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 512; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) s_l[threadIdx.x] += s_l[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *loss = s_l[0] * (double)scale;
}

// out[c] = sum_r x[r][c] (fixed order): 32 columns x 8 row-groups per block.
__global__ void __launch_bounds__(256) k_colsum(const __nv_bfloat16 *x, int rows, int cols, int ld, float *out)
{
    __shared__ float s[8][33];
    const int c = blockIdx.x * 32 + threadIdx.x;
    float acc = 0.f;
    if (c < cols)
        for (int r = threadIdx.y; r < rows; r += 8) acc += __bfloat162float(x[(size_t)r * ld + c]);
    s[threadIdx.y][threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.y == 0 && c < cols) {
        float v = 0.f;
        for (int k = 0; k < 8; ++k) v += s[k][threadIdx.x];
        out[c] = v;
    }
}

// Adam (Kingma & Ba, 2015) with bias correction, step t >= 1.
__global__ void k_adam(float *p, const float *g, float *m, float *v, int n, float lr, float b1, float b2, float eps,
                       float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi; v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void k_lp_to_bf16(const float *p, __nv_bfloat16 *w1, __nv_bfloat16 *w2, __nv_bfloat16 *w3)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kMlpHid * kMlpInPad) w1[i] = __float2bfloat16_rn(p[kPadW1 + i]);
    if (i < kMlpHid * kMlpHid) w2[i] = __float2bfloat16_rn(p[kPadW2 + i]);
    if (i < kMlpOutPad * kMlpHid) w3[i] = __float2bfloat16_rn(p[kPadW3 + i]);
}

// The inference path's forward pass over rows of x ([n][16] bf16) -> out
// ([n][20] fp32); for checks of the fused network against other evaluations.
__global__ void __launch_bounds__(kLpThreads, 1) k_lp_forward(const LpWeights w, const __nv_bfloat16 *x, int n,
                                                               float *out)
{
    extern __shared__ __align__(16) unsigned char smem[];
    LpSmemWeights &W = *reinterpret_cast<LpSmemWeights *>(smem);
    LpWarpBuf &buf = reinterpret_cast<LpWarpBuf *>(smem + sizeof(LpSmemWeights))[threadIdx.x >> 5];
    lp_stage_weights(w, W);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * kLpWarps;
    for (int base = (blockIdx.x * kLpWarps + (threadIdx.x >> 5)) * 32; base < n; base += warps * 32) {
        const int i = base + lane;
        uint4 v0 = make_uint4(0u, 0u, 0u, 0u), v1 = v0;
        if (i < n) {
            v0 = reinterpret_cast<const uint4 *>(x + (size_t)i * kMlpInPad)[0];
            v1 = reinterpret_cast<const uint4 *>(x + (size_t)i * kMlpInPad)[1];
        }
        reinterpret_cast<uint4 *>(buf.x + lane * kLdx)[0] = v0;
        reinterpret_cast<uint4 *>(buf.x + lane * kLdx)[1] = v1;
        __syncwarp();
        lp_warp_forward(W, buf);
        if (i < n) {
            const float *orow = lp_out_rows(buf) + lane * kLdo;
            for (int k = 0; k < kMlpOut; ++k) out[(size_t)i * kMlpOut + k] = orow[k];
        }
        __syncwarp();
    }
}

int grid_1d(long long n, int threads) { return (int)((n + threads - 1) / threads); }

}  // namespace

size_t lp_sweep_smem_bytes() { return sizeof(LpSmemWeights) + kLpWarps * sizeof(LpWarpBuf); }

int lp_sweep_blocks(long long max_items, int R, int num_sms)
{
    long long b = (max_items + kLpThreads - 1) / kLpThreads;
    if (b > num_sms) b = num_sms;
    const long long need = (R + kLpThreads - 1) / kLpThreads;
    if (b < need) b = need;
    return (int)(b < 1 ? 1 : b);
}

cudaError_t lp_configure(int device)
{
    (void)device;
    const int bytes = (int)lp_sweep_smem_bytes();
    static_assert(sizeof(LpSmemWeights) % 16 == 0, "warp buffers must stay 16-byte aligned");
    static_assert(4 * kLpThreads * sizeof(double) + kLpThreads * sizeof(unsigned int) <=
                      kLpWarps * sizeof(LpWarpBuf), "reduction scratch must fit in the warp buffers");
    cudaError_t e = cudaFuncSetAttribute(k_sweep_lp<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_sweep_lp<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_sweep_lp<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_sweep_lp<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_lp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    return e;
}

// Virtual 128-thread blocks of the tcgen05 sweep: a multiple of kTcGroups, at
// most one CTA (kTcGroups groups) per SM.
int lp_tc_sweep_blocks(long long max_items, int R, int num_sms)
{
    long long b = (max_items + kTcRows - 1) / kTcRows;
    if (b > (long long)kTcGroups * num_sms) b = (long long)kTcGroups * num_sms;
    const long long need = (R + kTcRows - 1) / kTcRows;
    if (b < need) b = need;
    if (b < 1) b = 1;
    return (int)((b + kTcGroups - 1) / kTcGroups * kTcGroups);
}

cudaError_t lp_tc_sweep_configure()
{
    using Sm = TcSmemG<kTcGroups>;
    const int bytes = (int)sizeof(Sm);
    static_assert(sizeof(TcTile) >= kTcRows * (4 * sizeof(double) + sizeof(unsigned int)), "scratch");
    static_assert(sizeof(Sm) <= 227 * 1024, "shared memory");
    cudaError_t e = cudaFuncSetAttribute(k_sweep_lp_tc<kTcGroups, false, false>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_sweep_lp_tc<kTcGroups, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_sweep_lp_tc<kTcGroups, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_sweep_lp_tc<kTcGroups, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    return e;
}

// `blocks` counts virtual 128-thread blocks (a multiple of kTcGroups).
cudaError_t launch_sweep_lp_tc(const LpSweepArgs &a, bool hb, bool hd, int blocks, double *part,
                               unsigned long long *part_rej, int slots, int *err, cudaStream_t st)
{
    if (blocks % kTcGroups) return cudaErrorInvalidValue;
    const size_t sm = sizeof(TcSmemG<kTcGroups>);
    const int grid = blocks / kTcGroups, nt = kTcRows * kTcGroups;
    if (hb && hd) k_sweep_lp_tc<kTcGroups, true, true><<<grid, nt, sm, st>>>(a, part, part_rej, slots, err);
    else if (hb) k_sweep_lp_tc<kTcGroups, true, false><<<grid, nt, sm, st>>>(a, part, part_rej, slots, err);
    else if (hd) k_sweep_lp_tc<kTcGroups, false, true><<<grid, nt, sm, st>>>(a, part, part_rej, slots, err);
    else k_sweep_lp_tc<kTcGroups, false, false><<<grid, nt, sm, st>>>(a, part, part_rej, slots, err);
    return cudaGetLastError();
}

cudaError_t launch_sweep_lp(const LpSweepArgs &a, bool hb, bool hd, int blocks, cudaStream_t st)
{
    const size_t sm = lp_sweep_smem_bytes();
    if (hb && hd) k_sweep_lp<true, true><<<blocks, kLpThreads, sm, st>>>(a);
    else if (hb) k_sweep_lp<true, false><<<blocks, kLpThreads, sm, st>>>(a);
    else if (hd) k_sweep_lp<false, true><<<blocks, kLpThreads, sm, st>>>(a);
    else k_sweep_lp<false, false><<<blocks, kLpThreads, sm, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_lp_collect(const LpCollectArgs &a, bool hb, bool hd, int max_blocks, cudaStream_t st)
{
    if (a.count <= 0) return cudaSuccess;
    int blocks = grid_1d(a.count, 256);
    if (blocks > max_blocks) blocks = max_blocks;
    if (hb && hd) k_lp_collect<true, true><<<blocks, 256, 0, st>>>(a);
    else if (hb) k_lp_collect<true, false><<<blocks, 256, 0, st>>>(a);
    else if (hd) k_lp_collect<false, true><<<blocks, 256, 0, st>>>(a);
    else k_lp_collect<false, false><<<blocks, 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_gemm(const GemmArgs &g, bool ta, bool tb, cudaStream_t st)
{
    if (g.M <= 0 || g.N <= 0 || g.K <= 0) return cudaSuccess;
    if ((g.M | g.N | g.K | g.lda | g.ldb) & 7) return cudaErrorInvalidValue;
    if ((reinterpret_cast<uintptr_t>(g.A) | reinterpret_cast<uintptr_t>(g.B)) & 15) return cudaErrorInvalidValue;
    const dim3 grid((g.N + kGn - 1) / kGn, (g.M + kGm - 1) / kGm);
    if (!ta && !tb) k_gemm_bf16<false, false><<<grid, 128, 0, st>>>(g);
    else if (!ta && tb) k_gemm_bf16<false, true><<<grid, 128, 0, st>>>(g);
    else if (ta && tb) k_gemm_bf16<true, true><<<grid, 128, 0, st>>>(g);
    else k_gemm_bf16<true, false><<<grid, 128, 0, st>>>(g);
    return cudaGetLastError();
}

cudaError_t launch_lp_gather(const __nv_bfloat16 *x_all, const float *t_all, long long n_all, int batch,
                             uint64_t seed, uint64_t step, __nv_bfloat16 *xb, float *tb, cudaStream_t st)
{
    if (n_all <= 0 || batch <= 0) return cudaErrorInvalidValue;
    k_lp_gather<<<grid_1d(batch, 256), 256, 0, st>>>(x_all, t_all, n_all, batch, (uint32_t)seed,
                                                      (uint32_t)(seed >> 32), (uint32_t)step,
                                                      (uint32_t)(step >> 32), xb, tb);
    return cudaGetLastError();
}

cudaError_t launch_lp_head(const float *o, const float *t, int n_real, int n_rows, float scale, __nv_bfloat16 *d_o,
                           double *loss, cudaStream_t st)
{
    k_lp_head<<<1, 1024, 0, st>>>(o, t, n_real, n_rows, scale, d_o, loss);
    return cudaGetLastError();
}

cudaError_t launch_colsum(const __nv_bfloat16 *x, int rows, int cols, int ld, float *out, cudaStream_t st)
{
    k_colsum<<<(cols + 31) / 32, dim3(32, 8), 0, st>>>(x, rows, cols, ld, out);
    return cudaGetLastError();
}

cudaError_t launch_adam(float *p, const float *g, float *m, float *v, int n, float lr, float b1, float b2, float eps,
                        long long t, cudaStream_t st)
{
    const float c1 = 1.f - powf(b1, (float)t), c2 = 1.f - powf(b2, (float)t);
    k_adam<<<grid_1d(n, 256), 256, 0, st>>>(p, g, m, v, n, lr, b1, b2, eps, c1, c2);
    return cudaGetLastError();
}

cudaError_t launch_lp_to_bf16(const float *p, __nv_bfloat16 *w1, __nv_bfloat16 *w2, __nv_bfloat16 *w3,
                              cudaStream_t st)
{
    k_lp_to_bf16<<<grid_1d(kMlpHid * kMlpHid, 256), 256, 0, st>>>(p, w1, w2, w3);
    return cudaGetLastError();
}

cudaError_t launch_lp_forward(const LpWeights &w, const __nv_bfloat16 *x, int n, float *out, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    int blocks = (n + kLpThreads - 1) / kLpThreads;
    if (blocks > 1024) blocks = 1024;
    k_lp_forward<<<blocks, kLpThreads, lp_sweep_smem_bytes(), st>>>(w, x, n, out);
    return cudaGetLastError();
}

}  // namespace esp
