// Monte Carlo kernels for sm_103a.
//
//   k_sweep_ell      one colour class of a Metropolis sweep, every replica
//                    (metropolis + delta_energy_get, get_quant.F90:52-182,264-337)
//   k_energy_part    energy_get (get_quant.F90:186-261) and sum_i s_i per
//                    replica: per-block partials into scratch ...
//   k_energy_reduce  ... reduced in a fixed order (deterministic FP64)
//   k_local_terms    the per-site linear/quadratic coefficients (parity checks)
//   k_obs_part       orderparam_get / staggered_get sums (get_quant.F90:366-422),
//                    reduced by k_energy_reduce
//   k_sc_part        spincorr_get (get_quant.F90:495-540) bin sums per
//                    replica, reduced by k_sc_reduce, accumulated by k_sc_finish
//   k_sf_part        mcarlo_structure_factor (get_quant.F90:649-717): F(q) per
//                    replica; k_sf_finish projects and accumulates per slot
//   k_measure        per-measurement accumulators and binning
//                    (mcarlo.F90:536-590, pt.F90:789-849)
//   k_pm_hist        Pm_get (get_quant.F90:425-493) as an integer histogram
//   k_pt_swap        pt_swap (pt.F90:1235-1288) on temperature labels
//   k_init_spins     ferro / rand start configurations (mcarlo.F90:271-293)
//   k_spins_in/out   spin_matrix(3,N,slots) <-> the permuted FP32 SoA state
//
// Layout: spins are FP32 SoA (sx, sy, sz), element (p, r) at p*R + r, with p
// the colour-major permuted site index and r the replica.  Consecutive threads
// take consecutive replicas of one site, so spin loads and stores of a warp
// are contiguous and the table entries of a site are read once per warp.
#include "esp_device.cuh"
#include "esp_kernels.h"

namespace esp {

// ---------------------------------------------------------------------------
// Per-block partial sums, no atomics.  Thread t of block b works on replica
// (b*blockDim + t) % R for the whole launch, so the threads of one replica in
// a block are t0, t0+R, ...; thread t < slots (= min(R, blockDim)) sums them
// and adds the result to its block's own slot part[b][t].  Every launch of the
// sweep uses the same grid, so slot (b, t) always belongs to the same block and
// the same replica; k_fold later sums the slots of each replica in block order
// (deterministic) into the running totals.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void add_block_slots(float e, float mx, float my, float mz, unsigned int nrej,
                                                int R, int slots, double *part, unsigned long long *part_rej)
{
    __shared__ double s_part[256][4];
    __shared__ unsigned int s_rej[256];
    const int t = threadIdx.x;
    const int nt = blockDim.x;
    const size_t slot = (size_t)blockIdx.x * slots + t;
    if (R >= nt) {
        double *o = part + 4 * slot;
        o[0] += (double)e; o[1] += (double)mx; o[2] += (double)my; o[3] += (double)mz;
        part_rej[slot] += (unsigned long long)nrej;
        return;
    }
    s_part[t][0] = (double)e; s_part[t][1] = (double)mx; s_part[t][2] = (double)my; s_part[t][3] = (double)mz;
    s_rej[t] = nrej;
    __syncthreads();
    if (t < R) {
        double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
        unsigned long long nr = 0;
        for (int u = t; u < nt; u += R) {
            a0 += s_part[u][0]; a1 += s_part[u][1]; a2 += s_part[u][2]; a3 += s_part[u][3];
            nr += s_rej[u];
        }
        double *o = part + 4 * slot;
        o[0] += a0; o[1] += a1; o[2] += a2; o[3] += a3;
        part_rej[slot] += nr;
    }
}

// Sum every block's slot of replica r, add it to the running energy /
// magnetisation and to the rejected counter of r's temperature slot, and
// clear the slots.  One block per replica: thread t takes blocks t, t+256, ...
// and a fixed-shape tree combines the threads, so the sum is deterministic.
__global__ void __launch_bounds__(256) k_fold(FoldArgs a)
{
    __shared__ double s_v[4][256];
    __shared__ unsigned long long s_n[256];
    const int r = blockIdx.x;
    double e = 0, mx = 0, my = 0, mz = 0;
    unsigned long long nr = 0;
    for (int b = threadIdx.x; b < a.nblocks; b += blockDim.x) {
        long long t = ((long long)r - (long long)b * a.block_threads) % a.R;
        if (t < 0) t += a.R;
        if (t >= a.slots) continue;
        const size_t slot = (size_t)b * a.slots + t;
        double *o = a.part + 4 * slot;
        e += o[0]; mx += o[1]; my += o[2]; mz += o[3];
        o[0] = 0.0; o[1] = 0.0; o[2] = 0.0; o[3] = 0.0;
        nr += a.part_rej[slot];
        a.part_rej[slot] = 0ull;
    }
    const int t = threadIdx.x;
    s_v[0][t] = e; s_v[1][t] = mx; s_v[2][t] = my; s_v[3][t] = mz; s_n[t] = nr;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (t < w) {
            for (int c = 0; c < 4; ++c) s_v[c][t] += s_v[c][t + w];
            s_n[t] += s_n[t + w];
        }
        __syncthreads();
    }
    if (t == 0) {
        a.e_run[r] += s_v[0][0];
        a.m_run[3 * r] += s_v[1][0]; a.m_run[3 * r + 1] += s_v[2][0]; a.m_run[3 * r + 2] += s_v[3][0];
        a.rej[2 * a.temp_of[r] + a.phase] += s_n[0];
    }
}

// ---------------------------------------------------------------------------
// One colour class, all replicas.  Grid-stride with a stride that is a
// multiple of R, so each thread keeps one replica for its whole life.
// ---------------------------------------------------------------------------
template <bool HB, bool HD>
__global__ void __launch_bounds__(256) k_sweep_ell(const SweepArgs a)
{
    const int R = a.R;
    const long long nthreads = (long long)gridDim.x * blockDim.x;
    const long long S = (nthreads / R) * R;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = tid < S;
    const int r = (int)(tid % R);
    const int temp = a.temp_of[r];
    // FP32 per thread (a few updates each); FP64 from the block sums on
    float accE = 0.f, accX = 0.f, accY = 0.f, accZ = 0.f;
    unsigned int nrej = 0;
    uint32_t sw_lo, sw_hi;
    sweep_index(a, sw_lo, sw_hi);
    if (live) {
        const float beta = a.beta[temp];
        const int pstep = (int)(S / R);
        const bool has_si = a.si != nullptr, has_f = a.fld != nullptr;
        for (int pi = (int)(tid / R); pi < a.n_c; pi += pstep) {
            const int p = a.off_c + pi;
            const size_t idx = (size_t)p * R + r;
            const float ox = a.sx[idx], oy = a.sy[idx], oz = a.sz[idx];
            float gx = 0.f, gy = 0.f, gz = 0.f;
            float qxx = 0.f, qyy = 0.f, qzz = 0.f, qxy = 0.f, qxz = 0.f, qyz = 0.f;
            // entries come in groups of 8 (the host pads every list with
            // zero-coupling entries pointing at the site itself), so each
            // group issues 8 independent index loads and then 24 spin loads
            const int nn = __ldg(a.nnb + p);
            for (int k0 = 0; k0 < nn; k0 += 8) {
                int q[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) q[j] = __ldg(a.nbr + (size_t)(k0 + j) * a.N + p);
                float tx[8], ty[8], tz[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const size_t iq = (size_t)q[j] * R + r;
                    tx[j] = __ldg(a.sx + iq); ty[j] = __ldg(a.sy + iq); tz[j] = __ldg(a.sz + iq);
                }
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const size_t e = (size_t)(k0 + j) * a.N + p;
                    const float J = __ldg(a.J + e);
                    gx = fmaf(-J, tx[j], gx); gy = fmaf(-J, ty[j], gy); gz = fmaf(-J, tz[j], gz);
                    if (HB) bq_form(__ldg(a.B + e), tx[j], ty[j], tz[j], qxx, qyy, qzz, qxy, qxz, qyz);
                    // s_k x D_ik (the DM term of delta_energy_get as s_i . (s_k x D))
                    if (HD) dm_field(__ldg(a.Dx + e), __ldg(a.Dy + e), __ldg(a.Dz + e), tx[j], ty[j], tz[j], gx, gy, gz);
                }
            }
            const int orig = __ldg(a.perm + p);
            if (has_si || has_f) {
                const int at = orig % a.num_atoms;
                if (has_si) si_form(__ldg(a.si + at), qxx, qyy, qzz, qxy, qxz, qyz);
                if (has_f) {
                    const float4 f = __ldg(a.fld + at);
                    gx = __fadd_rn(gx, f.x); gy = __fadd_rn(gy, f.y); gz = __fadd_rn(gz, f.z);
                }
            }
            const Philox4 x = philox4x32_10((uint32_t)orig, (uint32_t)r, sw_lo, sw_hi, a.key0, a.key1);
            float nx, ny, nz;
            trial_spin(a.mode, a.tilt, __ldg(a.mag + p), ox, oy, oz, x.x, x.y, nx, ny, nz);
            const float dx = nx - ox, dy = ny - oy, dz = nz - oz;
            // s_new^T Q s_new - s_old^T Q s_old = d^T Q (s_new + s_old)
            const float de = delta_energy(HB || has_si, gx, gy, gz, qxx, qyy, qzz, qxy, qxz, qyz, ox, oy, oz, nx, ny, nz);
            const bool acc = metropolis_accept(beta, de, x.z);
            if (acc) {
                a.sx[idx] = nx; a.sy[idx] = ny; a.sz[idx] = nz;
                accE += de;
                accX += dx; accY += dy; accZ += dz;
            } else {
                ++nrej;
            }
        }
    }
    add_block_slots(accE, accX, accY, accZ, nrej, R, a.slots, a.part, a.part_rej);
}

// ---------------------------------------------------------------------------
// Direct energy and magnetisation, stage 1: thread-local FP64 sums of the
// per-site energies e_i = 1/2 sum_k pair_ik + Delta (s.a)^2 + f.s, then a
// fixed-order block reduction per replica into scratch[block][R][4].
// ---------------------------------------------------------------------------
struct EnergyArgs {
    const int32_t *nnb, *nbr;
    const float *J, *B, *Dx, *Dy, *Dz;
    const int32_t *perm;
    const float4 *si, *fld;
    const float *sx, *sy, *sz;
    double *scratch;          // [gridDim.x][R][4]
    int32_t N, R, num_atoms;
};

// Per-replica sums of the four values in s_acc[t] of this block's threads
// (the replica of thread t is (blockIdx.x * blockDim.x + t) % R, threads at or
// past S hold nothing), in a fixed order, to scratch[block][R][4].
__device__ void store_block_replica_sums(double (*s_acc)[4], long long S, int R, double *scratch)
{
    const int t = threadIdx.x;
    const int base = (int)(((long long)blockIdx.x * blockDim.x) % R);
    for (int rr = t; rr < R; rr += blockDim.x) {
        // first thread of this block holding replica rr
        int u0 = rr - base;
        if (u0 < 0) u0 += R;
        double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
        for (int u = u0; u < (int)blockDim.x; u += R) {
            const long long g = (long long)blockIdx.x * blockDim.x + u;
            if (g >= S) break;
            a0 += s_acc[u][0]; a1 += s_acc[u][1]; a2 += s_acc[u][2]; a3 += s_acc[u][3];
        }
        double *o = scratch + ((size_t)blockIdx.x * R + rr) * 4;
        o[0] = a0; o[1] = a1; o[2] = a2; o[3] = a3;
    }
}

template <bool HB, bool HD>
__global__ void __launch_bounds__(256) k_energy_part(const EnergyArgs a)
{
    __shared__ double s_acc[256][4];
    const int R = a.R;
    const long long nthreads = (long long)gridDim.x * blockDim.x;
    const long long S = (nthreads / R) * R;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0, mx = 0, my = 0, mz = 0;
    if (tid < S) {
        const int r = (int)(tid % R);
        const int pstep = (int)(S / R);
        for (int p = (int)(tid / R); p < a.N; p += pstep) {
            const size_t idx = (size_t)p * R + r;
            const float ox = a.sx[idx], oy = a.sy[idx], oz = a.sz[idx];
            float pair = 0.f;
            const int nn = a.nnb[p];
            for (int k = 0; k < nn; ++k) {
                const size_t ee = (size_t)k * a.N + p;
                const size_t iq = (size_t)a.nbr[ee] * R + r;
                const float tx = a.sx[iq], ty = a.sy[iq], tz = a.sz[iq];
                const float d = ox * tx + oy * ty + oz * tz;
                pair -= a.J[ee] * d;
                if (HB) pair += a.B[ee] * d * d;
                if (HD) {
                    const float cx = oy * tz - oz * ty, cy = oz * tx - ox * tz, cz = ox * ty - oy * tx;
                    pair += a.Dx[ee] * cx + a.Dy[ee] * cy + a.Dz[ee] * cz;
                }
            }
            float site = 0.5f * pair;
            if (a.si || a.fld) {
                const int at = a.perm[p] % a.num_atoms;
                if (a.si) {
                    const float4 s = a.si[at];
                    const float sa = ox * s.x + oy * s.y + oz * s.z;
                    site += s.w * sa * sa;
                }
                if (a.fld) {
                    const float4 f = a.fld[at];
                    site += f.x * ox + f.y * oy + f.z * oz;
                }
            }
            e += (double)site;
            mx += (double)ox; my += (double)oy; mz += (double)oz;
        }
    }
    const int t = threadIdx.x;
    s_acc[t][0] = e; s_acc[t][1] = mx; s_acc[t][2] = my; s_acc[t][3] = mz;
    __syncthreads();
    store_block_replica_sums(s_acc, S, R, a.scratch);
}

// Stage 1 of the order-parameter / staggered sums: per (site, replica) the
// FP32 products s.a and c s, summed per thread and block in FP64 like the
// energy.
__global__ void __launch_bounds__(256) k_obs_part(const ObsArgs a)
{
    __shared__ double s_acc[256][4];
    const int R = a.R;
    const long long nthreads = (long long)gridDim.x * blockDim.x;
    const long long S = (nthreads / R) * R;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double op = 0, qx = 0, qy = 0, qz = 0;
    if (tid < S) {
        const int r = (int)(tid % R);
        const int pstep = (int)(S / R);
        for (int p = (int)(tid / R); p < a.N; p += pstep) {
            const size_t idx = (size_t)p * R + r;
            const float ox = a.sx[idx], oy = a.sy[idx], oz = a.sz[idx];
            const float4 w = __ldg(a.atom + a.perm[p] % a.num_atoms);
            float fo = 0.f, fx = 0.f, fy = 0.f, fz = 0.f;
            obs_add(ox, oy, oz, w, fo, fx, fy, fz);
            op += (double)fo; qx += (double)fx; qy += (double)fy; qz += (double)fz;
        }
    }
    const int t = threadIdx.x;
    s_acc[t][0] = op; s_acc[t][1] = qx; s_acc[t][2] = qy; s_acc[t][3] = qz;
    __syncthreads();
    store_block_replica_sums(s_acc, S, R, a.scratch);
}

// Stage 2: out_e[r] = sum over blocks, out_m[r][3] likewise.  One block per
// replica: thread t takes blocks t, t+256, ... and a fixed-shape tree combines
// the threads, so the sum is deterministic.
__global__ void __launch_bounds__(256) k_energy_reduce(const double *scratch, int nblocks, int R, double *out_e,
                                                       double *out_m)
{
    __shared__ double s_v[4][256];
    const int r = blockIdx.x, t = threadIdx.x;
    double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
    for (int b = t; b < nblocks; b += blockDim.x) {
        const double *o = scratch + ((size_t)b * R + r) * 4;
        a0 += o[0]; a1 += o[1]; a2 += o[2]; a3 += o[3];
    }
    s_v[0][t] = a0; s_v[1][t] = a1; s_v[2][t] = a2; s_v[3][t] = a3;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (t < w)
            for (int c = 0; c < 4; ++c) s_v[c][t] += s_v[c][t + w];
        __syncthreads();
    }
    if (t == 0) {
        out_e[r] = s_v[0][0];
        if (out_m) { out_m[3 * r] = s_v[1][0]; out_m[3 * r + 1] = s_v[2][0]; out_m[3 * r + 2] = s_v[3][0]; }
    }
}

// ---------------------------------------------------------------------------
// spincorr_get: bins in pairs per pass; per item (site, replica) FP32 sums over
// the bin's entries, FP64 per thread and block (like the energy).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_sc_part(const ScArgs a)
{
    __shared__ double s_acc[256][4];
    const int R = a.R, N = a.N;
    const long long nthreads = (long long)gridDim.x * blockDim.x;
    const long long S = (nthreads / R) * R;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int npass = (a.B + 1) / 2;
    for (int pass = 0; pass < npass; ++pass) {
        double v[4] = {0, 0, 0, 0};
        if (tid < S) {
            const int r = (int)(tid % R);
            const int pstep = (int)(S / R);
            for (int p = (int)(tid / R); p < N; p += pstep) {
                const size_t idx = (size_t)p * R + r;
                const float ox = a.sx[idx], oy = a.sy[idx], oz = a.sz[idx];
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    const int b = 2 * pass + q;
                    if (b < a.B) {
                        const int e0 = a.off[(size_t)b * N + p], e1 = a.off[(size_t)(b + 1) * N + p];
                        float sum = 0.f, sabs = 0.f;
                        for (int e = e0; e < e1; ++e) {
                            const size_t ee = (size_t)e * N + p;
                            const size_t iq = (size_t)a.nb[ee] * R + r;
                            const float d = ox * a.sx[iq] + oy * a.sy[iq] + oz * a.sz[iq];
                            const float wd = a.w[ee] * d;
                            sum += wd;
                            sabs += fabsf(wd);
                        }
                        v[2 * q] += (double)sum;
                        v[2 * q + 1] += (double)sabs;
                    }
                }
            }
        }
        const int t = threadIdx.x;
        s_acc[t][0] = v[0]; s_acc[t][1] = v[1]; s_acc[t][2] = v[2]; s_acc[t][3] = v[3];
        __syncthreads();
        store_block_replica_sums(s_acc, S, R, a.scratch + (size_t)pass * gridDim.x * R * 4);
        __syncthreads();
    }
}

// Block (r, pass): fixed-order sum of the blocks' partials of replica r.
__global__ void __launch_bounds__(256) k_sc_reduce(const double *scratch, int nblocks, int R, double *out)
{
    __shared__ double s_v[4][256];
    const int r = blockIdx.x, pass = blockIdx.y, t = threadIdx.x;
    const double *base = scratch + (size_t)pass * nblocks * R * 4;
    double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
    for (int b = t; b < nblocks; b += blockDim.x) {
        const double *o = base + ((size_t)b * R + r) * 4;
        a0 += o[0]; a1 += o[1]; a2 += o[2]; a3 += o[3];
    }
    s_v[0][t] = a0; s_v[1][t] = a1; s_v[2][t] = a2; s_v[3][t] = a3;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (t < w)
            for (int c = 0; c < 4; ++c) s_v[c][t] += s_v[c][t + w];
        __syncthreads();
    }
    if (t < 4) out[((size_t)pass * R + r) * 4 + t] = s_v[t][0];
}

// Per temperature slot: spincorr += S_b, spincorr_abs += A_b, tot_abs += |S_b|
// (get_quant.F90:535-537).
__global__ void k_sc_finish(const ScArgs a)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.R) return;
    const int r = a.repl_at[t];
    for (int b = 0; b < a.B; ++b) {
        const double *o = a.out + ((size_t)(b >> 1) * a.R + r) * 4 + 2 * (b & 1);
        double *acc = a.acc + ((size_t)t * a.B + b) * 3;
        acc[0] += o[0];
        acc[1] += o[1];
        acc[2] += fabs(o[0]);
    }
}

// ---------------------------------------------------------------------------
// Structure factor.  Block: 64 q-points x 4 replicas (thread = one pair);
// the block walks all sites in tiles of 64, staging the tile's phases
// e^{i q.r} (shared by the replicas) and spins (shared by the q-points) in
// shared memory.  FP32 sums; the phase is exact to 2^-24 of a turn.
// ---------------------------------------------------------------------------
constexpr int kSfQ = 64, kSfR = 4, kSfTile = 64;

__device__ __forceinline__ long long sf_step(const SfArgs &a)
{
    return a.step + (a.ctr ? (long long)*a.ctr : 0ll);
}

__global__ void __launch_bounds__(kSfQ * kSfR) k_sf_part(const SfArgs a)
{
    if (sf_step(a) % a.every != 0) return;
    __shared__ float2 s_ph[kSfTile][kSfQ];
    __shared__ float s_sp[kSfTile][kSfR][3];
    const int qi = threadIdx.x % kSfQ, rr = threadIdx.x / kSfQ;
    const int q = blockIdx.x * kSfQ + qi, r = blockIdx.y * kSfR + rr;
    float fxr = 0.f, fxi = 0.f, fyr = 0.f, fyi = 0.f, fzr = 0.f, fzi = 0.f;
    for (int i0 = 0; i0 < a.N; i0 += kSfTile) {
        __syncthreads();
        for (int k = threadIdx.x; k < kSfTile * kSfQ; k += blockDim.x) {
            const int j = k / kSfQ, qq = k % kSfQ;
            const int i = i0 + j, qg = blockIdx.x * kSfQ + qq;
            float c = 0.f, sn = 0.f;
            if (i < a.N && qg < a.nq) {
                const int4 n = __ldg(a.site_n + i);
                const float4 f = __ldg(a.site_f + i);
                const uint4 qfix = __ldg(a.q_fix + qg);
                const float4 qf = __ldg(a.q_frac + qg);
                // whole cells: exact modulo one turn in 32-bit fixed point
                const uint32_t t = qfix.x * (uint32_t)n.x + qfix.y * (uint32_t)n.y + qfix.z * (uint32_t)n.z;
                const float tw = (float)(int32_t)t * 2.3283064365386963e-10f;   // [-1/2, 1/2) turn
                float tf = qf.x * f.x + qf.y * f.y + qf.z * f.z;
                tf -= rintf(tf);
                sincospif(2.f * (tw + tf), &sn, &c);
            }
            s_ph[j][qq] = make_float2(c, sn);
        }
        for (int k = threadIdx.x; k < kSfTile * kSfR; k += blockDim.x) {
            const int j = k / kSfR, rq = k % kSfR;
            const int i = i0 + j, rg = blockIdx.y * kSfR + rq;
            float x = 0.f, y = 0.f, z = 0.f;
            if (i < a.N && rg < a.R) {
                const size_t idx = (size_t)__ldg(a.inv + i) * a.R + rg;
                x = a.sx[idx]; y = a.sy[idx]; z = a.sz[idx];
            }
            s_sp[j][rq][0] = x; s_sp[j][rq][1] = y; s_sp[j][rq][2] = z;
        }
        __syncthreads();
#pragma unroll 8
        for (int j = 0; j < kSfTile; ++j) {
            const float2 ph = s_ph[j][qi];
            const float x = s_sp[j][rr][0], y = s_sp[j][rr][1], z = s_sp[j][rr][2];
            fxr = fmaf(x, ph.x, fxr); fxi = fmaf(x, ph.y, fxi);
            fyr = fmaf(y, ph.x, fyr); fyi = fmaf(y, ph.y, fyi);
            fzr = fmaf(z, ph.x, fzr); fzi = fmaf(z, ph.y, fzi);
        }
    }
    if (q < a.nq && r < a.R) {
        float *o = a.fq + ((size_t)r * a.nq + q) * 6;
        o[0] = fxr; o[1] = fxi; o[2] = fyr; o[3] = fyi; o[4] = fzr; o[5] = fzi;
    }
}

// Per (q, slot): F_perp = F - q (q.F) / q.q, NSF = Re(p.F_perp) / |p|
// (get_quant.F90:693-710), accumulated in FP64.
__global__ void k_sf_finish(const SfArgs a)
{
    if (sf_step(a) % a.every != 0) return;
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k == 0) *a.count += 1;
    if (k >= (long long)a.nq * a.R) return;
    const int q = (int)(k % a.nq), t = (int)(k / a.nq);
    const float4 qc = __ldg(a.q_cart + q);
    if (qc.w != 0.f) return;
    const float *f = a.fq + ((size_t)a.repl_at[t] * a.nq + q) * 6;
    const double qx = qc.x, qy = qc.y, qz = qc.z;
    const double qq = qx * qx + qy * qy + qz * qz;
    const double dre = (f[0] * qx + f[2] * qy + f[4] * qz) / qq;
    const double dim = (f[1] * qx + f[3] * qy + f[5] * qz) / qq;
    const double xr = f[0] - dre * qx, xi = f[1] - dim * qx;
    const double yr = f[2] - dre * qy, yi = f[3] - dim * qy;
    const double zr = f[4] - dre * qz, zi = f[5] - dim * qz;
    const double f2 = xr * xr + xi * xi + yr * yr + yi * yi + zr * zr + zi * zi;
    const double nsf = (a.px * xr + a.py * yr + a.pz * zr) / a.pnorm;
    double *o = a.acc + ((size_t)t * a.nq + q) * 3;
    o[0] += f2;
    o[1] += f2 - nsf * nsf;
    o[2] += nsf * nsf;
}

// ---------------------------------------------------------------------------
// Local terms g_i (3) and Q_i (6) of every (site, replica), FP32.
// ---------------------------------------------------------------------------
template <bool HB, bool HD>
__global__ void k_local_terms(const EnergyArgs a, float *g, float *q)
{
    const long long total = (long long)a.N * a.R;
    for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < total;
         it += (long long)gridDim.x * blockDim.x) {
        const int p = (int)(it / a.R), r = (int)(it % a.R);
        float gx = 0, gy = 0, gz = 0, qxx = 0, qyy = 0, qzz = 0, qxy = 0, qxz = 0, qyz = 0;
        const int nn = a.nnb[p];
        for (int k = 0; k < nn; ++k) {
            const size_t e = (size_t)k * a.N + p;
            const size_t iq = (size_t)a.nbr[e] * a.R + r;
            const float tx = a.sx[iq], ty = a.sy[iq], tz = a.sz[iq];
            const float J = a.J[e];
            gx = fmaf(-J, tx, gx); gy = fmaf(-J, ty, gy); gz = fmaf(-J, tz, gz);
            if (HB) {
                const float Bv = a.B[e];
                const float bx = Bv * tx, by = Bv * ty, bz = Bv * tz;
                qxx = fmaf(bx, tx, qxx); qyy = fmaf(by, ty, qyy); qzz = fmaf(bz, tz, qzz);
                qxy = fmaf(bx, ty, qxy); qxz = fmaf(bx, tz, qxz); qyz = fmaf(by, tz, qyz);
            }
            if (HD) {
                const float dx = a.Dx[e], dy = a.Dy[e], dz = a.Dz[e];
                gx += ty * dz - tz * dy; gy += tz * dx - tx * dz; gz += tx * dy - ty * dx;
            }
        }
        if (a.si || a.fld) {
            const int at = a.perm[p] % a.num_atoms;
            if (a.si) {
                const float4 s = a.si[at];
                const float dx = s.w * s.x, dy = s.w * s.y, dz = s.w * s.z;
                qxx = fmaf(dx, s.x, qxx); qyy = fmaf(dy, s.y, qyy); qzz = fmaf(dz, s.z, qzz);
                qxy = fmaf(dx, s.y, qxy); qxz = fmaf(dx, s.z, qxz); qyz = fmaf(dy, s.z, qyz);
            }
            if (a.fld) { const float4 f = a.fld[at]; gx += f.x; gy += f.y; gz += f.z; }
        }
        float *go = g + (size_t)it * 3;
        go[0] = gx; go[1] = gy; go[2] = gz;
        float *qo = q + (size_t)it * 6;
        qo[0] = qxx; qo[1] = qyy; qo[2] = qzz; qo[3] = qxy; qo[4] = qxz; qo[5] = qyz;
    }
}

// ---------------------------------------------------------------------------
// Per-measurement accumulators, one thread per temperature slot.
// data[t][6] += E, E^2, E^4, |m|, m^2, m^4 with m = M/N (mcarlo.F90:536-543);
// binning sums as mcarlo.F90:548-590 (pt_quirk: pt.F90:841-849 divides a
// completed block by 2**l, l being the level's position).
// ---------------------------------------------------------------------------
__global__ void k_measure(MeasureArgs a)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.R) return;
    if (a.ctr) a.step += (long long)*a.ctr;
    const int r = a.repl_at[t];
    const double e = a.e_run[r];
    const double mx = a.m_run[3 * r] / (double)a.N;
    const double my = a.m_run[3 * r + 1] / (double)a.N;
    const double mz = a.m_run[3 * r + 2] / (double)a.N;
    const double m2 = mx * mx + my * my + mz * mz;
    const double ee = e * e;
    double *d = a.data + 6 * t;
    d[0] += e; d[1] += ee; d[2] += ee * ee;
    const double am = sqrt(m2);
    d[3] += am; d[4] += m2; d[5] += m2 * m2;
    if (a.series) {
        double *o = a.series + (((a.step - 1) % a.series_cap) * a.R + t) * 2;
        o[0] = e; o[1] = am;
    }
    // orderparam_get / staggered_get of this replica (mcarlo.F90:553-568)
    double aop = 0.0, asm_ = 0.0;
    if (a.obs) {
        double *od = a.obs_data + 6 * t;
        const double *q = a.obs_rep + a.R + 3 * r;
        if (a.obs & 1) {
            const double op = a.obs_rep[r] / (double)a.N;
            const double o2 = op * op;
            aop = sqrt(o2);
            od[0] += aop; od[1] += o2; od[2] += o2 * o2;
        }
        if (a.obs & 2) {
            const double qx = q[0] / (double)a.N, qy = q[1] / (double)a.N, qz = q[2] / (double)a.N;
            const double q2 = qx * qx + qy * qy + qz * qz;
            asm_ = sqrt(q2);
            od[3] += asm_; od[4] += q2; od[5] += q2 * q2;
        }
    }
    if (a.nlev > 0) {
        double *ls = a.lsum + (size_t)t * a.nlev * 2;
        double *bn = a.binning + (size_t)t * a.nlev * 2;
        double *ols = a.obs ? a.obs_lsum + (size_t)t * a.nlev * 2 : nullptr;
        double *obn = a.obs ? a.obs_bin + (size_t)t * a.nlev * 2 : nullptr;
        for (int l = 0; l < a.nlev; ++l) {
            ls[2 * l] += e / (double)a.N;
            ls[2 * l + 1] += am;
            if (ols) { ols[2 * l] += aop; ols[2 * l + 1] += asm_; }
            const long long blk = 1LL << a.levels[l];
            if (a.step % blk == 0) {
                const double div = a.pt_quirk ? (double)(1LL << (l + 1)) : (double)blk;
                for (int c = 0; c < 2; ++c) {
                    const double v = ls[2 * l + c] / div;
                    bn[2 * l + c] += v * v;
                    ls[2 * l + c] = 0.0;
                    if (ols) {
                        const double w = ols[2 * l + c] / div;
                        obn[2 * l + c] += w * w;
                        ols[2 * l + c] = 0.0;
                    }
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// P(M) histogram (Pm_get): per unit cell |sum_atoms s| -> bin
// max(nint((|m| - m_min)/(m_max - m_min) * (nf-1)) + 1, 1), counted as
// integers per temperature slot (the reference adds 1/d_m = 100 per hit).
// Block: a tile of cells x all replicas, shared histogram [R][nf] when it fits.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_pm_hist(PmArgs a)
{
    // block (x, y): a chunk of cells x the replica tile [y*rt, y*rt + nrt)
    // per replica of the tile: histograms [nh][nf], P(M) then P(OP), P(SM)
    extern __shared__ unsigned int s_hist[];
    const int R = a.R, nf = a.nf;
    const int nh = a.obs ? 3 : 1;
    const int r0 = blockIdx.y * a.rt;
    const int nrt = min(a.rt, R - r0);
    for (int i = threadIdx.x; i < nrt * nh * nf; i += blockDim.x) s_hist[i] = 0u;
    __syncthreads();
    const float m_min = (float)a.m_min, scale = (float)((double)(nf - 1) / (a.m_max - a.m_min));
    const long long total = (long long)a.ncell * nrt;
    for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < total;
         it += (long long)gridDim.x * blockDim.x) {
        const int cell = (int)(it / nrt), rr = (int)(it % nrt), r = r0 + rr;
        float mx = 0.f, my = 0.f, mz = 0.f, op = 0.f, qx = 0.f, qy = 0.f, qz = 0.f;
        for (int at = 0; at < a.num_atoms; ++at) {
            const int p = __ldg(a.inv + cell * a.num_atoms + at);
            const size_t idx = (size_t)p * R + r;
            const float sx = a.sx[idx], sy = a.sy[idx], sz = a.sz[idx];
            mx += sx; my += sy; mz += sz;
            if (a.obs) obs_add(sx, sy, sz, __ldg(a.obs_atom + at), op, qx, qy, qz);
        }
        unsigned int *hr = s_hist + (size_t)rr * nh * nf;
        if (a.count_m) atomicAdd(hr + (pm_bin(mx, my, mz, m_min, scale, nf) - 1), 1u);
        if (a.obs & 1) atomicAdd(hr + nf + (pm_bin_value(op, m_min, scale, nf) - 1), 1u);
        if (a.obs & 2) atomicAdd(hr + 2 * nf + (pm_bin(qx, qy, qz, m_min, scale, nf) - 1), 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nrt * nh * nf; i += blockDim.x) {
        const unsigned int c = s_hist[i];
        if (c) {
            const int rr = i / (nh * nf), k = (i / nf) % nh, f = i % nf;
            const int t = a.temp_of[r0 + rr];
            if (k == 0) atomicAdd(a.counts + (size_t)t * nf + f, (unsigned long long)c);
            else atomicAdd(a.obs_counts + ((size_t)t * 2 + (k - 1)) * nf + f, (unsigned long long)c);
        }
    }
}

// ---------------------------------------------------------------------------
// pt_swap on labels: pairs (a, a+1), a = start0, start0+2, ...; one thread.
// x = (1/T_a - 1/T_{a+1}) (E_a - E_{a+1}) with the running energies; accept
// if x > 0 or u < exp(x).  The replicas keep their spins; the slot->replica
// map (the reference's `map`) and replica->slot map are exchanged.
// ---------------------------------------------------------------------------
__global__ void k_pt_swap(PtSwapArgs a)
{
    // pairs are disjoint, one thread each; slots form groups of `group`
    // consecutive temperatures (independent lattices) and pairs never cross
    // a group boundary
    uint32_t idx_lo = a.idx_lo, idx_hi = a.idx_hi;
    int start0 = a.start0;
    if (a.ctr) {
        const unsigned long long idx = (((unsigned long long)a.idx_hi << 32) | a.idx_lo) + a.ctr[1];
        idx_lo = (uint32_t)idx; idx_hi = (uint32_t)(idx >> 32);
        start0 = (int)((a.ctr[3] + (unsigned long long)a.unit_off + 1ull) % 2ull);
    }
    const int per_group = a.group / 2;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int g = i / per_group, k = i % per_group;
    if (g >= a.R / a.group) return;
    const int sl = start0 + 2 * k;
    if (sl + 1 >= a.group) return;
    const int s = g * a.group + sl;
    const int ra = a.repl_at[s], rb = a.repl_at[s + 1];
    const double x = (a.inv_t[s] - a.inv_t[s + 1]) * (a.e_run[ra] - a.e_run[rb]);
    a.num_swaps[2 * s] += 1;
    a.num_swaps[2 * (s + 1)] += 1;
    bool swap = x > 0.0;
    if (!swap) {
        const Philox4 v = philox4x32_10((uint32_t)s, idx_lo, idx_hi, 0xFFFFFFFFu, a.key0, a.key1);
        swap = u53(v.x, v.y) < exp(x);
    }
    if (swap) {
        a.repl_at[s] = rb; a.repl_at[s + 1] = ra;
        a.temp_of[rb] = s; a.temp_of[ra] = s + 1;
        a.num_swaps[2 * s + 1] += 1;
        a.num_swaps[2 * (s + 1) + 1] += 1;
    }
}

// ---------------------------------------------------------------------------
// Start configurations: kind 0 ferro (0,0,m); kind 1 rand with
// theta = pi*u1, phi = 2 pi*u2 (mcarlo.F90:279-293), one configuration for
// all replicas as pt.F90:448-459 does.
// ---------------------------------------------------------------------------
// spin_matrix(3, N, t0 .. t0+nt-1) in FP64 (reference site order, slot t
// holding replica repl_at[t]) -> the FP32 state, and back.  One thread per
// (slot, site, component) of the staged block, reading or writing it
// contiguously.
__global__ void k_spins_in(const double *stage, const int32_t *inv, const int32_t *repl_at, float *sx, float *sy,
                           float *sz, int N, int R, int t0, int nt)
{
    const long long total = 3LL * N * nt;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(k % 3);
        const long long ti = k / 3;
        const int i = (int)(ti % N), t = t0 + (int)(ti / N);
        const size_t o = (size_t)inv[i] * R + repl_at[t];
        float *dst = c == 0 ? sx : (c == 1 ? sy : sz);
        dst[o] = (float)stage[k];
    }
}

__global__ void k_spins_out(double *stage, const int32_t *inv, const int32_t *repl_at, const float *sx,
                            const float *sy, const float *sz, int N, int R, int t0, int nt)
{
    const long long total = 3LL * N * nt;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(k % 3);
        const long long ti = k / 3;
        const int i = (int)(ti % N), t = t0 + (int)(ti / N);
        const size_t o = (size_t)inv[i] * R + repl_at[t];
        const float *src = c == 0 ? sx : (c == 1 ? sy : sz);
        stage[k] = (double)src[o];
    }
}

__global__ void k_init_spins(const int32_t *perm, const float *mag, float *sx, float *sy, float *sz,
                             int N, int R, int kind, uint32_t k0, uint32_t k1)
{
    const long long total = (long long)N * R;
    for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < total;
         it += (long long)gridDim.x * blockDim.x) {
        const int p = (int)(it / R);
        const float m = mag[p];
        float x = 0.f, y = 0.f, z = m;
        if (kind == 1) {
            const Philox4 v = philox4x32_10((uint32_t)perm[p], 0xFFFFFFFEu, 0u, 0u, k0, k1);
            const double u1 = (double)v.x * (1.0 / 4294967296.0), u2 = (double)v.y * (1.0 / 4294967296.0);
            double st, ct, sp, cp;
            sincospi(u1, &st, &ct);
            sincospi(2.0 * u2, &sp, &cp);
            x = (float)(m * st * cp); y = (float)(m * st * sp); z = (float)(m * ct);
        }
        sx[it] = x; sy[it] = y; sz[it] = z;
    }
}

// ---------------------------------------------------------------------------
// Host-side launchers
// ---------------------------------------------------------------------------
static int grid_for(long long items, int threads, int max_blocks)
{
    long long b = (items + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > max_blocks) b = max_blocks;
    return (int)b;
}

int sweep_blocks(long long max_items, int R, int max_blocks)
{
    const int threads = 256;
    int blocks = grid_for(max_items, threads, max_blocks);
    // the stride must hold at least one copy of every replica
    const int need = (R + threads - 1) / threads;
    return blocks < need ? need : blocks;
}

cudaError_t launch_fold(const FoldArgs &a, cudaStream_t st)
{
    k_fold<<<a.R, 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_sweep(const SweepArgs &a, bool hb, bool hd, int blocks, cudaStream_t st)
{
    const int threads = 256;
    if (hb && hd) k_sweep_ell<true, true><<<blocks, threads, 0, st>>>(a);
    else if (hb) k_sweep_ell<true, false><<<blocks, threads, 0, st>>>(a);
    else if (hd) k_sweep_ell<false, true><<<blocks, threads, 0, st>>>(a);
    else k_sweep_ell<false, false><<<blocks, threads, 0, st>>>(a);
    return cudaGetLastError();
}

int energy_blocks(int N, int R, int max_blocks)
{
    const int threads = 256;
    int blocks = grid_for((long long)N * R, threads, max_blocks);
    const int need = (R + threads - 1) / threads;
    return blocks < need ? need : blocks;
}

cudaError_t launch_energy(const EnergyArgsHost &h, double *out_e, double *out_m, int blocks, cudaStream_t st)
{
    EnergyArgs a;
    a.nnb = h.nnb; a.nbr = h.nbr; a.J = h.J; a.B = h.B; a.Dx = h.Dx; a.Dy = h.Dy; a.Dz = h.Dz;
    a.perm = h.perm; a.si = h.si; a.fld = h.fld; a.sx = h.sx; a.sy = h.sy; a.sz = h.sz;
    a.scratch = h.scratch; a.N = h.N; a.R = h.R; a.num_atoms = h.num_atoms;
    const bool hb = h.B != nullptr, hd = h.Dx != nullptr;
    if (hb && hd) k_energy_part<true, true><<<blocks, 256, 0, st>>>(a);
    else if (hb) k_energy_part<true, false><<<blocks, 256, 0, st>>>(a);
    else if (hd) k_energy_part<false, true><<<blocks, 256, 0, st>>>(a);
    else k_energy_part<false, false><<<blocks, 256, 0, st>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_energy_reduce<<<h.R, 256, 0, st>>>(h.scratch, blocks, h.R, out_e, out_m);
    return cudaGetLastError();
}

cudaError_t launch_obs(const ObsArgs &a, double *out_op, double *out_sm, int blocks, cudaStream_t st)
{
    k_obs_part<<<blocks, 256, 0, st>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_energy_reduce<<<a.R, 256, 0, st>>>(a.scratch, blocks, a.R, out_op, out_sm);
    return cudaGetLastError();
}

cudaError_t launch_spincorr(const ScArgs &a, int blocks, cudaStream_t st)
{
    if (a.B <= 0) return cudaSuccess;
    k_sc_part<<<blocks, 256, 0, st>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_sc_reduce<<<dim3(a.R, (a.B + 1) / 2), 256, 0, st>>>(a.scratch, blocks, a.R, a.out);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    k_sc_finish<<<(a.R + 127) / 128, 128, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_sfactor(const SfArgs &a, cudaStream_t st)
{
    if (a.nq <= 0) return cudaSuccess;
    k_sf_part<<<dim3((a.nq + kSfQ - 1) / kSfQ, (a.R + kSfR - 1) / kSfR), kSfQ * kSfR, 0, st>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const long long n = (long long)a.nq * a.R;
    k_sf_finish<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_local_terms(const EnergyArgsHost &h, float *g, float *q, cudaStream_t st)
{
    EnergyArgs a;
    a.nnb = h.nnb; a.nbr = h.nbr; a.J = h.J; a.B = h.B; a.Dx = h.Dx; a.Dy = h.Dy; a.Dz = h.Dz;
    a.perm = h.perm; a.si = h.si; a.fld = h.fld; a.sx = h.sx; a.sy = h.sy; a.sz = h.sz;
    a.scratch = nullptr; a.N = h.N; a.R = h.R; a.num_atoms = h.num_atoms;
    const int blocks = grid_for((long long)h.N * h.R, 256, 4096);
    const bool hb = h.B != nullptr, hd = h.Dx != nullptr;
    if (hb && hd) k_local_terms<true, true><<<blocks, 256, 0, st>>>(a, g, q);
    else if (hb) k_local_terms<true, false><<<blocks, 256, 0, st>>>(a, g, q);
    else if (hd) k_local_terms<false, true><<<blocks, 256, 0, st>>>(a, g, q);
    else k_local_terms<false, false><<<blocks, 256, 0, st>>>(a, g, q);
    return cudaGetLastError();
}

cudaError_t launch_measure(const MeasureArgs &a, cudaStream_t st)
{
    k_measure<<<(a.R + 127) / 128, 128, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_pm(const PmArgs &a0, int max_blocks, cudaStream_t st)
{
    PmArgs a = a0;
    // replica tile: its [rt][nh][nf] histograms fit in 96 KB of shared memory
    const size_t cap = 96 * 1024;
    const int nh = a.obs ? 3 : 1;
    a.rt = (int)(cap / ((size_t)nh * a.nf * sizeof(unsigned int)));
    if (a.rt < 1) return cudaErrorInvalidValue;
    if (a.rt > a.R) a.rt = a.R;
    a.use_shared = 1;
    static bool attr_set[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (!attr_set[dev]) {
        e = cudaFuncSetAttribute(k_pm_hist, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cap);
        if (e != cudaSuccess) return e;
        attr_set[dev] = true;
    }
    const int tiles = (a.R + a.rt - 1) / a.rt;
    // few blocks, many items each: the flush of the block histograms is a
    // global atomic per non-empty bin, so fewer blocks means less contention
    const int cap_blocks = max_blocks / 8 / tiles > 0 ? max_blocks / 8 / tiles : 1;
    int bx = grid_for((long long)a.ncell * a.rt, 256, cap_blocks);
    const size_t smem = (size_t)a.rt * nh * a.nf * sizeof(unsigned int);
    k_pm_hist<<<dim3(bx, tiles), 256, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_pt_swap(const PtSwapArgs &a, cudaStream_t st)
{
    if (a.group < 2 || a.R % a.group != 0) return a.group == 1 ? cudaSuccess : cudaErrorInvalidValue;
    const int threads = (a.R / a.group) * (a.group / 2);
    k_pt_swap<<<(threads + 127) / 128, 128, 0, st>>>(a);
    return cudaGetLastError();
}

__global__ void k_bump(unsigned long long *ctr, unsigned long long d0, unsigned long long d1, unsigned long long d2,
                       unsigned long long d3)
{
    ctr[0] += d0; ctr[1] += d1; ctr[2] += d2; ctr[3] += d3;
}

cudaError_t launch_bump(unsigned long long *ctr, const unsigned long long d[4], cudaStream_t st)
{
    k_bump<<<1, 1, 0, st>>>(ctr, d[0], d[1], d[2], d[3]);
    return cudaGetLastError();
}

cudaError_t launch_spins_in(const double *stage, const int32_t *inv, const int32_t *repl_at, float *sx, float *sy,
                            float *sz, int N, int R, int t0, int nt, cudaStream_t st)
{
    const int blocks = grid_for(3LL * N * nt, 256, 4096);
    k_spins_in<<<blocks, 256, 0, st>>>(stage, inv, repl_at, sx, sy, sz, N, R, t0, nt);
    return cudaGetLastError();
}

cudaError_t launch_spins_out(double *stage, const int32_t *inv, const int32_t *repl_at, const float *sx,
                             const float *sy, const float *sz, int N, int R, int t0, int nt, cudaStream_t st)
{
    const int blocks = grid_for(3LL * N * nt, 256, 4096);
    k_spins_out<<<blocks, 256, 0, st>>>(stage, inv, repl_at, sx, sy, sz, N, R, t0, nt);
    return cudaGetLastError();
}

cudaError_t launch_init_spins(const int32_t *perm, const float *mag, float *sx, float *sy, float *sz,
                              int N, int R, int kind, uint64_t seed, cudaStream_t st)
{
    const int blocks = grid_for((long long)N * R, 256, 4096);
    k_init_spins<<<blocks, 256, 0, st>>>(perm, mag, sx, sy, sz, N, R, kind, (uint32_t)seed,
                                         (uint32_t)(seed >> 32));
    return cudaGetLastError();
}

}  // namespace esp
