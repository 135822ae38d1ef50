// Cluster-resident sweeps for translation-invariant periodic lattices.
//
// One thread-block cluster holds one replica's whole lattice in distributed
// shared memory for the length of a launch: each CTA of the cluster owns a
// slab of z planes, stored class-major (parity class k = atom*8 + px*4 + py*2
// + pz, then half-cell coordinates), so a colour pass (a set of classes) reads
// its neighbours from its own or a peer CTA's shared memory and writes only its
// own.  A launch runs `n_meas` units of `steps_measure` sweeps, each unit
// followed by the measurement of mcarlo.F90:536-590 / pt.F90:789-849
// (accumulators, binning, Pm_get histogram), all without touching global
// memory; each CTA reads its slab at the start and writes it back at the end
// as one contiguous block (k_to_slabs / k_from_slabs convert the spin arrays
// around the launch).
//
// Updates, random numbers and the local-field arithmetic are those of
// k_sweep_ell (same colouring, same Philox counter (site, replica, sweep), the
// stencil lists in the merged-list order, the shared explicitly rounded
// trial / field / energy functions), so both kernels produce the same
// trajectory.  Waits are cluster barriers only (hardware, no spinning).
#include <cooperative_groups.h>
#include <type_traits>

#include "esp_cluster.h"
#include "esp_device.cuh"

namespace cg = cooperative_groups;

namespace esp {

// NT threads per CTA and S sites per thread in a colour pass: 512 x 1 (one
// CTA per SM), 256 x 1 (two per SM), or 512 x 2, whose threads update two
// sites of a colour with interleaved instruction streams (fewer, evenly
// loaded passes when a colour holds between 1 and 2 times 512 sites).  All
// within 128 registers per thread: a sub-partition of the SM that holds four
// warps has 16,384 registers for them.
// Warp-aggregated increments of a shared-memory histogram (1-based bins,
// bin <= 0 adds nothing; every lane of the warp calls together).  Low
// temperatures put almost every cell in one bin: while a warp's 32 cells share
// one bin, and the same bin as its previous call, the count stays in a
// register (one atomic per run instead of one per call); mixed warps add per
// lane.
struct WarpRun {
    int bin = -1;
    unsigned cnt = 0u;
};
__device__ __forceinline__ void hist_add(unsigned *h, WarpRun &run, int bin)
{
    const int b0 = __shfl_sync(0xffffffffu, bin, 0);
    if (__all_sync(0xffffffffu, bin == b0)) {
        if (b0 == run.bin) {
            run.cnt += 32u;
            return;
        }
        if ((threadIdx.x & 31) == 0 && run.bin > 0) atomicAdd(h + (run.bin - 1), run.cnt);
        run.bin = b0;
        run.cnt = 32u;
    } else if (bin > 0) {
        atomicAdd(h + (bin - 1), 1u);
    }
}
__device__ __forceinline__ void hist_flush(unsigned *h, const WarpRun &run)
{
    if ((threadIdx.x & 31) == 0 && run.bin > 0) atomicAdd(h + (run.bin - 1), run.cnt);
}

// HB, HD: the lattice has biquadratic / DM couplings (a.has_b, a.has_d), as
// compile-time flags so the neighbour loop carries no tests for absent terms.
template <int NT, int S, bool HB, bool HD>
__global__ void __launch_bounds__(NT, NT > 256 ? 1 : 2) k_sweep_cluster(const ClusterArgs a)
{
    static_assert(NT % 32 == 0 && NT <= 640, "the reduction scratch holds at most 20 warps");
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    const int csize = (int)cluster.num_blocks();
    const int r = blockIdx.x / csize;  // replica of this cluster
    const int Hx = a.Lx >> 1, Hy = a.Ly >> 1;
    const int Hzl = slab_planes(a.pz, a.nA, rank) >> 1;   // half planes of this CTA
    const int per_class = Hx * Hy * Hzl;
    const int n_local = per_class * a.nclass;
    const int z0 = slab_z0(a.pz, a.nA, rank);
    const size_t site0 = (size_t)(z0 >> 1) * Hx * Hy * a.nclass;   // sites of the ranks before this one
    const FastDiv fd_pc = rank < a.nA ? a.fd_pc : a.fd_pc2;
    const unsigned long long sweep_base = a.sweep_base + (a.ctr ? a.ctr[0] : 0ull);
    const long long meas_base = a.meas_base + (a.ctr ? (long long)a.ctr[2] : 0ll);

    // shared memory: stencil copy | histograms P(M) [, P(OP), P(SM)] |
    // reduction scratch | spins (stencil_words is a multiple of 4, so every
    // part stays 16-byte aligned)
    extern __shared__ __align__(16) unsigned char smem[];
    ClusterStencil *st = reinterpret_cast<ClusterStencil *>(smem);
    const ClusterNbr *nbt = reinterpret_cast<const ClusterNbr *>(st + 1);
    unsigned int *hist = reinterpret_cast<unsigned int *>(smem) + a.stencil_words;
    const int nhist = a.obs ? 3 : 1;
    // reduction scratch: [0, 112) warp partials; [128, 144) a CTA's totals of
    // a measurement, two buffers by the measurement's parity; [144, 149) the
    // CTA's end-of-launch totals
    double *red = reinterpret_cast<double *>(hist + ((nhist * a.nf + 3) & ~3));
    // the slot's accumulators, kept by rank 0 for the launch (the slot of a
    // replica does not change inside a launch): data, obs data, binning
    // levels, binning sums and variances of E/N, |m| and of |OP|, |SM|
    double *acc = red + kClusterRedDoubles;
    double *c_data = acc, *c_odata = acc + 6;
    int *c_lev = reinterpret_cast<int *>(acc + 12);
    double *c_ls = acc + 12 + kClusterMaxLev / 2, *c_bn = c_ls + 2 * kClusterMaxLev;
    double *c_ols = c_bn + 2 * kClusterMaxLev, *c_obn = c_ols + 2 * kClusterMaxLev;
    float *s3 = reinterpret_cast<float *>(acc + kClusterAccDoubles);   // [n_local][x, y, z]

    // ---- set-up: stencil and own spins -------------------------------------
    {
        const int *src = reinterpret_cast<const int *>(a.stencil);
        int *dst = reinterpret_cast<int *>(st);
        for (int i = threadIdx.x; i < a.stencil_words; i += blockDim.x) dst[i] = src[i];
        for (int i = threadIdx.x; i < nhist * a.nf; i += blockDim.x) hist[i] = 0u;
    }
    // this CTA's slab: one contiguous block of 3 n_local floats, or gathered
    // from the spin arrays
    float *slab = a.slab ? a.slab + ((size_t)r * a.N + site0) * 3 : nullptr;
    auto slab_global = [&](int l) -> size_t {
        int k, rem, q1, hx, hy, hzl;
        fdivmod(l, fd_pc, k, rem);
        fdivmod(rem, a.fd_hx, q1, hx);
        fdivmod(q1, a.fd_hy, hzl, hy);
        const int at = k >> 3, px = (k >> 2) & 1, py = (k >> 1) & 1, pz = k & 1;
        const int x = 2 * hx + px, y = 2 * hy + py, z = z0 + 2 * hzl + pz;
        return (size_t)__ldg(a.inv + ((z * a.Ly + y) * a.Lx + x) * a.na + at) * a.R + r;
    };
    if (slab) {
        for (int i = threadIdx.x; i < 3 * n_local; i += blockDim.x) s3[i] = slab[i];
    } else {
        for (int l = threadIdx.x; l < n_local; l += blockDim.x) {
            const size_t g = slab_global(l);
            s3[3 * l] = a.sx[g]; s3[3 * l + 1] = a.sy[g]; s3[3 * l + 2] = a.sz[g];
        }
    }
    const int temp = a.temp_of[r];
    const bool cache = a.measure && a.nlev <= kClusterMaxLev;
    if (rank == 0 && cache) {
        const int nl2 = 2 * a.nlev;
        for (int i = threadIdx.x; i < 6; i += blockDim.x) {
            c_data[i] = a.data[6 * temp + i];
            c_odata[i] = a.obs ? a.obs_data[6 * temp + i] : 0.0;
        }
        for (int i = threadIdx.x; i < a.nlev; i += blockDim.x) c_lev[i] = a.levels[i];
        for (int i = threadIdx.x; i < nl2; i += blockDim.x) {
            c_ls[i] = a.lsum[(size_t)temp * nl2 + i];
            c_bn[i] = a.binning[(size_t)temp * nl2 + i];
            c_ols[i] = a.obs ? a.obs_lsum[(size_t)temp * nl2 + i] : 0.0;
            c_obn[i] = a.obs ? a.obs_bin[(size_t)temp * nl2 + i] : 0.0;
        }
    }
    cluster.sync();

    const float beta = a.beta[temp];
    // sums of the per-sweep FP32 sums since the last measurement, as float pairs
    F2 accE{0.f, 0.f}, accX{0.f, 0.f}, accY{0.f, 0.f}, accZ{0.f, 0.f};
    unsigned long long nrej = 0;
    const float pm_scale = (float)((double)(a.nf - 1) / (a.m_max - a.m_min));
    // replica totals, held by thread 0 of rank 0
    double e_run = 0.0, m_run[3] = {0.0, 0.0, 0.0};
    if (rank == 0 && threadIdx.x == 0) {
        e_run = a.e_run[r];
        m_run[0] = a.m_run[3 * r]; m_run[1] = a.m_run[3 * r + 1]; m_run[2] = a.m_run[3 * r + 2];
    }

    // Metropolis updates of the sites of items its[0..SN) of a colour pass
    // (class_order from c0): local field from the stencil, trial, test
    // (metropolis, get_quant.F90:52-182, delta_energy_get :264-337), each
    // site's arithmetic in the same order as k_sweep_ell
    auto update = [&](auto snc, const int (&its)[decltype(snc)::value], int c0, uint32_t sw_lo, uint32_t sw_hi,
                      float &fE, float &fX, float &fY, float &fZ) {
        constexpr int SN = decltype(snc)::value;
        int l[SN], at[SN], orig[SN];
        float ox[SN], oy[SN], oz[SN];
        float gx[SN], gy[SN], gz[SN], qxx[SN], qyy[SN], qzz[SN], qxy[SN], qxz[SN], qyz[SN];
        const ClusterNbr *nb[SN];
        const uint4 *tab[SN];
        int cnt_k = 0;
#pragma unroll
        for (int s = 0; s < SN; ++s) {
            int ci, rem, q1, hx, hy, hzl;
            fdivmod(its[s], fd_pc, ci, rem);
            const int k = st->class_order[c0 + ci];
            l[s] = k * per_class + rem;
            fdivmod(rem, a.fd_hx, q1, hx);
            fdivmod(q1, a.fd_hy, hzl, hy);
            at[s] = k >> 3;
            const int px = (k >> 2) & 1, py = (k >> 1) & 1, pzb = k & 1;
            const int x = 2 * hx + px, y = 2 * hy + py, z = z0 + 2 * hzl + pzb;
            orig[s] = ((z * a.Ly + y) * a.Lx + x) * a.na + at[s];
            ox[s] = s3[3 * l[s]]; oy[s] = s3[3 * l[s] + 1]; oz[s] = s3[3 * l[s] + 2];
            gx[s] = gy[s] = gz[s] = 0.f;
            qxx[s] = qyy[s] = qzz[s] = qxy[s] = qxz[s] = qyz[s] = 0.f;
            // neighbour e of site l from the precomputed table shared by every
            // replica's cluster, four entries per 16-byte word: the local
            // index, with bit 31 set and the owner rank in bits 24-30 when the
            // neighbour lives in a peer CTA; lists are padded to multiples of
            // 8 with zero-coupling self entries
            cnt_k = st->count[k];   // equal for the SN sites
            nb[s] = nbt + k * st->maxst;
            tab[s] = reinterpret_cast<const uint4 *>(a.nbidx) + (size_t)(st->maxst >> 2) * site0 + l[s];
        }
        // a batch of NB neighbours of every site: read from this CTA's shared
        // memory when every lane of the warp finds all of them here (warps
        // cover slab planes, so this is the common case), else through the
        // cluster window
        auto batch = [&](auto nbc, int e0) {
            constexpr int NB = decltype(nbc)::value;
            constexpr int NQ = (NB + 3) / 4;
            uint32_t id[SN][4 * NQ];
#pragma unroll
            for (int s = 0; s < SN; ++s)
#pragma unroll
                for (int j = 0; j < NQ; ++j) {
                    const uint4 w = __ldg(tab[s] + (size_t)((e0 >> 2) + j) * n_local);
                    id[s][4 * j] = w.x; id[s][4 * j + 1] = w.y; id[s][4 * j + 2] = w.z; id[s][4 * j + 3] = w.w;
                }
            float tx[SN][NB], ty[SN][NB], tz[SN][NB];
            uint32_t any_remote = 0u;
#pragma unroll
            for (int s = 0; s < SN; ++s)
#pragma unroll
                for (int j = 0; j < NB; ++j) any_remote |= id[s][j];
            if (__all_sync(__activemask(), (any_remote >> 31) == 0u)) {
#pragma unroll
                for (int s = 0; s < SN; ++s)
#pragma unroll
                    for (int j = 0; j < NB; ++j) {
                        const float *p = s3 + 3 * id[s][j];
                        tx[s][j] = p[0]; ty[s][j] = p[1]; tz[s][j] = p[2];
                    }
            } else {
#pragma unroll
                for (int s = 0; s < SN; ++s)
#pragma unroll
                    for (int j = 0; j < NB; ++j) {
                        const uint32_t v = id[s][j];
                        const float *p = (v >> 31) ? cluster.map_shared_rank(s3, (int)((v >> 24) & 0x7fu)) : s3;
                        p += 3 * (v & 0xffffffu);
                        tx[s][j] = p[0]; ty[s][j] = p[1]; tz[s][j] = p[2];
                    }
            }
#pragma unroll
            for (int s = 0; s < SN; ++s)
#pragma unroll
                for (int j = 0; j < NB; ++j) {
                    const ClusterNbr &se = nb[s][e0 + j];
                    const float J = se.J;
                    gx[s] = fmaf(-J, tx[s][j], gx[s]); gy[s] = fmaf(-J, ty[s][j], gy[s]); gz[s] = fmaf(-J, tz[s][j], gz[s]);
                    if (HB)
                        bq_form(se.B, tx[s][j], ty[s][j], tz[s][j], qxx[s], qyy[s], qzz[s], qxy[s], qxz[s], qyz[s]);
                    if (HD) dm_field(se.Dx, se.Dy, se.Dz, tx[s][j], ty[s][j], tz[s][j], gx[s], gy[s], gz[s]);
                }
        };
        int e0 = 0;
        for (; e0 + 8 <= cnt_k; e0 += 8) batch(std::integral_constant<int, 8>{}, e0);
        // the last partial batch at its exact size (no padding work)
        switch (cnt_k - e0) {
        case 1: batch(std::integral_constant<int, 1>{}, e0); break;
        case 2: batch(std::integral_constant<int, 2>{}, e0); break;
        case 3: batch(std::integral_constant<int, 3>{}, e0); break;
        case 4: batch(std::integral_constant<int, 4>{}, e0); break;
        case 5: batch(std::integral_constant<int, 5>{}, e0); break;
        case 6: batch(std::integral_constant<int, 6>{}, e0); break;
        case 7: batch(std::integral_constant<int, 7>{}, e0); break;
        default: break;
        }
        float nx[SN], ny[SN], nz[SN], de[SN];
        bool acc[SN];
#pragma unroll
        for (int s = 0; s < SN; ++s) {
            if (a.has_si) si_form(st->si[at[s]], qxx[s], qyy[s], qzz[s], qxy[s], qxz[s], qyz[s]);
            if (a.has_f) {
                const float4 f = st->fld[at[s]];
                gx[s] = __fadd_rn(gx[s], f.x); gy[s] = __fadd_rn(gy[s], f.y); gz[s] = __fadd_rn(gz[s], f.z);
            }
            const Philox4 xr = philox4x32_10((uint32_t)orig[s], (uint32_t)r, sw_lo, sw_hi, a.key0, a.key1);
            trial_spin(a.mode, a.tilt, st->mag[at[s]], ox[s], oy[s], oz[s], xr.x, xr.y, nx[s], ny[s], nz[s]);
            const float d = delta_energy(HB || a.has_si, gx[s], gy[s], gz[s], qxx[s], qyy[s], qzz[s], qxy[s],
                                         qxz[s], qyz[s], ox[s], oy[s], oz[s], nx[s], ny[s], nz[s]);
            de[s] = d;
            acc[s] = metropolis_accept(beta, d, xr.z);
        }
#pragma unroll
        for (int s = 0; s < SN; ++s) {
            if (acc[s]) {
                s3[3 * l[s]] = nx[s]; s3[3 * l[s] + 1] = ny[s]; s3[3 * l[s] + 2] = nz[s];
                fE += de[s];
                fX += nx[s] - ox[s]; fY += ny[s] - oy[s]; fZ += nz[s] - oz[s];
            } else {
                ++nrej;
            }
        }
    };

    // Rank 0's warp 0 folds measurement m (the CTAs' totals in buffer m & 1)
    // into the replica totals and the accumulators of mcarlo.F90:536-590 for
    // this temperature slot: lane 0 the sums, one binning level per lane.
    auto fold_measurement = [&](const int m) {
        // lane 0 folds the CTAs' sums into the replica totals and the
        // accumulators of mcarlo.F90:536-590 for this temperature
        // slot; the binning levels, independent of one another, go
        // one per lane
        const double rn_inv = a.rn_inv;
        const long long step = meas_base + m + 1;
        double e = 0.0, am = 0.0, aop = 0.0, asm_ = 0.0;
        if (threadIdx.x == 0) {
            double d4[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            for (int q = 0; q < csize; ++q) {
                const double *pr = cluster.map_shared_rank(red, q);
#pragma unroll
                for (int c = 0; c < 8; ++c) d4[c] += pr[128 + 8 * (m & 1) + c];
            }
            e_run += d4[0];
            m_run[0] += d4[1]; m_run[1] += d4[2]; m_run[2] += d4[3];
            e = e_run;
            const double mx = m_run[0] * rn_inv, my = m_run[1] * rn_inv, mz = m_run[2] * rn_inv;
            const double m2 = mx * mx + my * my + mz * mz;
            const double ee = e * e;
            am = sqrt(m2);
            double *d = cache ? c_data : a.data + 6 * temp;
            d[0] += e; d[1] += ee; d[2] += ee * ee;
            d[3] += am; d[4] += m2; d[5] += m2 * m2;
            if (a.series) {
                double *o = a.series + (((step - 1) % a.series_cap) * a.R + temp) * 2;
                o[0] = e; o[1] = am;
            }
            // orderparam_get / staggered_get (mcarlo.F90:553-568)
            if (a.obs) {
                double *od = cache ? c_odata : a.obs_data + 6 * temp;
                if (a.obs & 1) {
                    const double op = d4[4] * rn_inv;
                    const double o2 = op * op;
                    aop = sqrt(o2);
                    od[0] += aop; od[1] += o2; od[2] += o2 * o2;
                }
                if (a.obs & 2) {
                    const double qx = d4[5] * rn_inv, qy = d4[6] * rn_inv, qz = d4[7] * rn_inv;
                    const double q2 = qx * qx + qy * qy + qz * qz;
                    asm_ = sqrt(q2);
                    od[3] += asm_; od[4] += q2; od[5] += q2 * q2;
                }
            }
        }
        if (a.nlev > 0) {
            e = __shfl_sync(0xffffffffu, e, 0);
            am = __shfl_sync(0xffffffffu, am, 0);
            aop = __shfl_sync(0xffffffffu, aop, 0);
            asm_ = __shfl_sync(0xffffffffu, asm_, 0);
        }
        for (int lv = threadIdx.x; lv < a.nlev; lv += 32) {
            const size_t g2 = ((size_t)temp * a.nlev + lv) * 2;
            double *ls = cache ? c_ls + 2 * lv : a.lsum + g2;
            double *bn = cache ? c_bn + 2 * lv : a.binning + g2;
            double *ols = !a.obs ? nullptr : (cache ? c_ols + 2 * lv : a.obs_lsum + g2);
            double *obn = !a.obs ? nullptr : (cache ? c_obn + 2 * lv : a.obs_bin + g2);
            ls[0] += e * rn_inv;
            ls[1] += am;
            if (ols) { ols[0] += aop; ols[1] += asm_; }
            const int lev = cache ? c_lev[lv] : a.levels[lv];
            const long long blk = 1LL << lev;
            if ((step & (blk - 1)) == 0) {
                // 1/2^n is exact, so the product equals the division
                const double inv_div = ldexp(1.0, -(a.pt_quirk ? lv + 1 : lev));
                for (int c = 0; c < 2; ++c) {
                    const double v2 = ls[c] * inv_div;
                    bn[c] += v2 * v2;
                    ls[c] = 0.0;
                    if (ols) {
                        const double w2 = ols[c] * inv_div;
                        obn[c] += w2 * w2;
                        ols[c] = 0.0;
                    }
                }
            }
        }
    };
    int pending = -1;   // measurement whose totals wait for rank 0's fold

    for (int m = 0; m < a.n_meas; ++m) {
        for (int sm = 0; sm < a.steps_measure; ++sm) {
            const unsigned long long sweep = sweep_base + (unsigned long long)m * a.steps_measure + sm;
            const uint32_t sw_lo = (uint32_t)sweep, sw_hi = (uint32_t)(sweep >> 32);
            // FP32 sums of one sweep, added to the FP64 ones after it
            float fE = 0.f, fX = 0.f, fY = 0.f, fZ = 0.f;
            for (int c = 0; c < st->ncolour; ++c) {
                const int c0 = st->colour_start[c];
                const int items = (st->colour_start[c + 1] - c0) * per_class;
                // S sites of the colour per thread, updated together (their
                // instruction streams interleave); a thread whose sites have
                // different stencil lengths, or that has one site left,
                // updates them one at a time
                for (int it0 = threadIdx.x; it0 < items; it0 += S * NT) {
                    int its[S];
#pragma unroll
                    for (int s = 0; s < S; ++s) its[s] = it0 + s * NT;
                    if constexpr (S == 1) {
                        update(std::integral_constant<int, 1>{}, its, c0, sw_lo, sw_hi, fE, fX, fY, fZ);
                    } else {
                        bool together = its[S - 1] < items;
                        if (together) {
                            const int cnt0 = st->count[st->class_order[c0 + its[0] / per_class]];
#pragma unroll
                            for (int s = 1; s < S; ++s)
                                together = together && st->count[st->class_order[c0 + its[s] / per_class]] == cnt0;
                        }
                        if (together) {
                            update(std::integral_constant<int, S>{}, its, c0, sw_lo, sw_hi, fE, fX, fY, fZ);
                        } else {
#pragma unroll
                            for (int s = 0; s < S; ++s)
                                if (its[s] < items) {
                                    const int one[1] = {its[s]};
                                    update(std::integral_constant<int, 1>{}, one, c0, sw_lo, sw_hi, fE, fX, fY, fZ);
                                }
                        }
                    }
                }
                cluster.sync();
                if (pending >= 0) {
                    if (rank == 0 && threadIdx.x < 32) fold_measurement(pending);
                    pending = -1;
                }
            }
            accE = f2_add(accE, fE); accX = f2_add(accX, fX); accY = f2_add(accY, fY); accZ = f2_add(accZ, fZ);
        }
        if (!a.measure) continue;
        // ---- measurement: cluster-wide sums of dE and dM (and, with the
        // optional measurements, of s.a and c s over the slab) ---------------
        {
            // float pairs within the CTA for dE and dM (FP64 is a slow pipe
            // on this GPU), plain FP32 for the order-parameter sums, FP64
            // across CTAs and into the running totals
            F2 p4[4] = {accE, accX, accY, accZ};
            accE = accX = accY = accZ = F2{0.f, 0.f};
            float v[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            if (a.obs) {
                float op = 0.f, qx = 0.f, qy = 0.f, qz = 0.f;
                for (int l = threadIdx.x; l < n_local; l += blockDim.x) {
                    int k, rem;
                    fdivmod(l, fd_pc, k, rem);
                    obs_add(s3[3 * l], s3[3 * l + 1], s3[3 * l + 2], __ldg(a.obs_atom + (k >> 3)), op, qx, qy, qz);
                }
                v[4] = op; v[5] = qx; v[6] = qy; v[7] = qz;
            }
#pragma unroll
            for (int c = 0; c < 4; ++c)
                for (int o = 16; o > 0; o >>= 1) p4[c] = f2_add(p4[c], f2_shfl_down(p4[c], o));
            if (a.obs) {
#pragma unroll
                for (int c = 4; c < 8; ++c)
                    for (int o = 16; o > 0; o >>= 1) v[c] += __shfl_down_sync(0xffffffffu, v[c], o);
            }
            const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
            // [warp][12] floats in the first 96 doubles: 4 pairs, 4 floats
            float *redf = reinterpret_cast<float *>(red);
            if (lane == 0) {
#pragma unroll
                for (int c = 0; c < 4; ++c) { redf[12 * warp + 2 * c] = p4[c].hi; redf[12 * warp + 2 * c + 1] = p4[c].lo; }
#pragma unroll
                for (int c = 4; c < 8; ++c) redf[12 * warp + 4 + c] = v[c];
            }
            __syncthreads();
            if (warp == 0) {
                const int nw = (int)(blockDim.x >> 5);
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    F2 x = lane < nw ? F2{redf[12 * lane + 2 * c], redf[12 * lane + 2 * c + 1]} : F2{0.f, 0.f};
                    for (int o = 16; o > 0; o >>= 1) x = f2_add(x, f2_shfl_down(x, o));
                    if (lane == 0) red[128 + 8 * (m & 1) + c] = f2_to_double(x);   // this CTA's totals
                }
#pragma unroll
                for (int c = 4; c < 8; ++c) {
                    float x = lane < nw ? redf[12 * lane + 4 + c] : 0.f;
                    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
                    if (lane == 0) red[128 + 8 * (m & 1) + c] = (double)x;
                }
            }
            // P(M) [P(OP), P(SM)] of this CTA's cells
            if (a.na > 1 || a.obs) {
                // cells in the local layout's order: the cell of parity class
                // p (0..7) and half-coordinates rem holds, for every atom, the
                // site (at * 8 + p) * per_class + rem, i.e. at * cstride + cl
                const int ncells_local = per_class * 8;         // cells of the slab
                const int cstride = per_class * 8;
                const int cl_end = (ncells_local + 31) & ~31;   // whole warps take part in the vote
                WarpRun run_m, run_op, run_sm;
                for (int cl = threadIdx.x; cl < cl_end; cl += blockDim.x) {
                    int bin = -1, bin_op = -1, bin_sm = -1;
                    if (cl < ncells_local) {
                        float mx = 0.f, my = 0.f, mz = 0.f, op = 0.f, qx = 0.f, qy = 0.f, qz = 0.f;
                        for (int at = 0; at < a.na; ++at) {
                            const int l = at * cstride + cl;
                            const float ox = s3[3 * l], oy = s3[3 * l + 1], oz = s3[3 * l + 2];
                            mx += ox; my += oy; mz += oz;
                            if (a.obs) obs_add(ox, oy, oz, __ldg(a.obs_atom + at), op, qx, qy, qz);
                        }
                        if (a.na > 1) bin = pm_bin(mx, my, mz, (float)a.m_min, pm_scale, a.nf);
                        if (a.obs & 1) bin_op = pm_bin_value(op, (float)a.m_min, pm_scale, a.nf);
                        if (a.obs & 2) bin_sm = pm_bin(qx, qy, qz, (float)a.m_min, pm_scale, a.nf);
                    }
                    hist_add(hist, run_m, bin);
                    if (a.obs) {
                        hist_add(hist + a.nf, run_op, bin_op);
                        hist_add(hist + 2 * a.nf, run_sm, bin_sm);
                    }
                }
                hist_flush(hist, run_m);
                if (a.obs) {
                    hist_flush(hist + a.nf, run_op);
                    hist_flush(hist + 2 * a.nf, run_sm);
                }
            }
            // the totals of this measurement wait in buffer (m & 1) of every
            // CTA; rank 0 folds them after the next cluster barrier (the next
            // colour pass, or the end of the launch), so a measurement adds no
            // cluster barrier of its own
            pending = m;
        }
    }

    // ---- end of launch: totals, rejected counts, histogram, spins ----------
    {
        // warp 0 may still read the last measurement's warp partials, which
        // the warp partials below overwrite
        __syncthreads();
        double v[4] = {f2_to_double(accE), f2_to_double(accX), f2_to_double(accY), f2_to_double(accZ)};
        unsigned long long nr = nrej;
        for (int c = 0; c < 4; ++c)
            for (int o = 16; o > 0; o >>= 1) v[c] += __shfl_down_sync(0xffffffffu, v[c], o);
        for (int o = 16; o > 0; o >>= 1) nr += __shfl_down_sync(0xffffffffu, nr, o);
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        if (lane == 0) {
            for (int c = 0; c < 4; ++c) red[4 * warp + c] = v[c];
            reinterpret_cast<unsigned long long *>(red + 96)[warp] = nr;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double t4[4] = {0, 0, 0, 0};
            unsigned long long tn = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
                for (int c = 0; c < 4; ++c) t4[c] += red[4 * w + c];
                tn += reinterpret_cast<unsigned long long *>(red + 96)[w];
            }
            for (int c = 0; c < 4; ++c) red[144 + c] = t4[c];
            reinterpret_cast<unsigned long long *>(red)[148] = tn;
        }
        if (a.na > 1)
            for (int i = threadIdx.x; i < a.nf; i += blockDim.x)
                if (hist[i]) atomicAdd(a.pm_counts + (size_t)temp * a.nf + i, (unsigned long long)hist[i]);
        if (a.obs)
            for (int i = threadIdx.x; i < 2 * a.nf; i += blockDim.x)
                if (hist[a.nf + i]) atomicAdd(a.obs_pm + (size_t)temp * 2 * a.nf + i, (unsigned long long)hist[a.nf + i]);
        cluster.sync();
        // the launch's last measurement, then the sums since it
        if (pending >= 0 && rank == 0 && threadIdx.x < 32) fold_measurement(pending);
        if (rank == 0) __syncthreads();   // the fold's accumulator writes before the write-back below
        if (rank == 0 && threadIdx.x == 0) {
            double d4[4] = {0, 0, 0, 0};
            unsigned long long tn = 0;
            for (int q = 0; q < csize; ++q) {
                const double *pr = cluster.map_shared_rank(red, q);
                for (int c = 0; c < 4; ++c) d4[c] += pr[144 + c];
                tn += reinterpret_cast<const unsigned long long *>(pr)[148];
            }
            a.e_run[r] = e_run + d4[0];
            a.m_run[3 * r] = m_run[0] + d4[1];
            a.m_run[3 * r + 1] = m_run[1] + d4[2];
            a.m_run[3 * r + 2] = m_run[2] + d4[3];
            a.rej[2 * temp + a.phase] += tn;
        }
        if (rank == 0 && cache) {
            const int nl2 = 2 * a.nlev;
            for (int i = threadIdx.x; i < 6; i += blockDim.x) {
                a.data[6 * temp + i] = c_data[i];
                if (a.obs) a.obs_data[6 * temp + i] = c_odata[i];
            }
            for (int i = threadIdx.x; i < nl2; i += blockDim.x) {
                a.lsum[(size_t)temp * nl2 + i] = c_ls[i];
                a.binning[(size_t)temp * nl2 + i] = c_bn[i];
                if (a.obs) { a.obs_lsum[(size_t)temp * nl2 + i] = c_ols[i]; a.obs_bin[(size_t)temp * nl2 + i] = c_obn[i]; }
            }
        }
    }
    if (slab) {
        for (int i = threadIdx.x; i < 3 * n_local; i += blockDim.x) slab[i] = s3[i];
    } else {
        for (int l = threadIdx.x; l < n_local; l += blockDim.x) {
            const size_t g = slab_global(l);
            a.sx[g] = s3[3 * l]; a.sy[g] = s3[3 * l + 1]; a.sz[g] = s3[3 * l + 2];
        }
    }
    // peers may still read this CTA's shared memory until every CTA is done
    cluster.sync();
}

// Position p (spin-array row) of local site l of rank q.
__device__ __forceinline__ int slab_row(const SlabArgs &a, int q, int l)
{
    int k, rem, q1, hx, hy, hzl;
    fdivmod(l, q < a.nA ? a.fd_pc : a.fd_pc2, k, rem);
    fdivmod(rem, a.fd_hx, q1, hx);
    fdivmod(q1, a.fd_hy, hzl, hy);
    const int at = k >> 3, px = (k >> 2) & 1, py = (k >> 1) & 1, pz = k & 1;
    const int x = 2 * hx + px, y = 2 * hy + py, z = slab_z0(a.pz, a.nA, q) + 2 * hzl + pz;
    return __ldg(a.inv + ((z * a.Ly + y) * a.Lx + x) * a.na + at);
}

// Sites of rank q and the first of them in a replica's slab order.
__device__ __forceinline__ int slab_sites(const SlabArgs &a, int q)
{
    return (slab_planes(a.pz, a.nA, q) >> 1) * (a.Lx >> 1) * (a.Ly >> 1) * 8 * a.na;
}
__device__ __forceinline__ size_t slab_site0(const SlabArgs &a, int q)
{
    return (size_t)(slab_z0(a.pz, a.nA, q) >> 1) * (a.Lx >> 1) * (a.Ly >> 1) * 8 * a.na;
}

// grid (n_local / 32, cs, R / 32) rounded up, blocks of 32 x 8 threads
__global__ void __launch_bounds__(256) k_to_slabs(const SlabArgs a)
{
    __shared__ float t[3][32][33];   // [component][replica][site]
    __shared__ int rows[32];
    const int l0 = blockIdx.x * 32, q = blockIdx.y, r0 = blockIdx.z * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nl = slab_sites(a, q);
    const size_t s0 = slab_site0(a, q);
    if (ty == 0) rows[tx] = l0 + tx < nl ? slab_row(a, q, l0 + tx) : 0;
    __syncthreads();
    for (int j = ty; j < 32; j += 8)
        if (l0 + j < nl && r0 + tx < a.R) {
            const size_t g = (size_t)rows[j] * a.R + r0 + tx;
            t[0][tx][j] = a.sx[g]; t[1][tx][j] = a.sy[g]; t[2][tx][j] = a.sz[g];
        }
    __syncthreads();
    for (int j = ty; j < 32; j += 8)
        if (r0 + j < a.R && l0 + tx < nl) {
            float *o = a.slab + ((size_t)(r0 + j) * a.N + s0 + l0 + tx) * 3;
            o[0] = t[0][j][tx]; o[1] = t[1][j][tx]; o[2] = t[2][j][tx];
        }
}

__global__ void __launch_bounds__(256) k_from_slabs(const SlabArgs a)
{
    __shared__ float t[3][32][33];   // [component][replica][site]
    __shared__ int rows[32];
    const int l0 = blockIdx.x * 32, q = blockIdx.y, r0 = blockIdx.z * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nl = slab_sites(a, q);
    const size_t s0 = slab_site0(a, q);
    if (ty == 0) rows[tx] = l0 + tx < nl ? slab_row(a, q, l0 + tx) : 0;
    for (int j = ty; j < 32; j += 8)
        if (r0 + j < a.R && l0 + tx < nl) {
            const float *i = a.slab + ((size_t)(r0 + j) * a.N + s0 + l0 + tx) * 3;
            t[0][j][tx] = i[0]; t[1][j][tx] = i[1]; t[2][j][tx] = i[2];
        }
    __syncthreads();
    for (int j = ty; j < 32; j += 8)
        if (l0 + j < nl && r0 + tx < a.R) {
            const size_t g = (size_t)rows[j] * a.R + r0 + tx;
            a.sx[g] = t[0][tx][j]; a.sy[g] = t[1][tx][j]; a.sz[g] = t[2][tx][j];
        }
}

cudaError_t launch_to_slabs(const SlabArgs &a, cudaStream_t st)
{
    const dim3 grid((a.n_local + 31) / 32, a.cs, (a.R + 31) / 32), block(32, 8);
    k_to_slabs<<<grid, block, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_from_slabs(const SlabArgs &a, cudaStream_t st)
{
    const dim3 grid((a.n_local + 31) / 32, a.cs, (a.R + 31) / 32), block(32, 8);
    k_from_slabs<<<grid, block, 0, st>>>(a);
    return cudaGetLastError();
}

size_t cluster_smem_bytes(int n_local, int nf, int nhist, size_t stencil_bytes)
{
    return ((stencil_bytes + 15) & ~(size_t)15) + (size_t)((nhist * nf + 3) & ~3) * sizeof(unsigned int) +
           (size_t)(kClusterRedDoubles + kClusterAccDoubles) * sizeof(double) + (size_t)3 * n_local * sizeof(float);
}

namespace {

using ClusterKernel = void (*)(ClusterArgs);

template <bool HB, bool HD>
ClusterKernel cluster_kernel_t(int nt, int S)
{
    return nt == 256 ? k_sweep_cluster<256, 1, HB, HD>
                     : (S == 2 ? k_sweep_cluster<512, 2, HB, HD> : k_sweep_cluster<512, 1, HB, HD>);
}

ClusterKernel cluster_kernel(int nt, int S, bool hb, bool hd)
{
    return hb ? (hd ? cluster_kernel_t<true, true>(nt, S) : cluster_kernel_t<true, false>(nt, S))
              : (hd ? cluster_kernel_t<false, true>(nt, S) : cluster_kernel_t<false, false>(nt, S));
}

}  // namespace

bool cluster_threads_ok(int nt, int S) { return (nt == 256 && S == 1) || (nt == 512 && (S == 1 || S == 2)); }

cudaError_t cluster_configure(size_t smem, int csize, int nt, int S)
{
    if (!cluster_threads_ok(nt, S)) return cudaErrorInvalidValue;
    cudaError_t e = cudaSuccess;
    for (int v = 0; v < 4 && e == cudaSuccess; ++v) {
        const ClusterKernel k = cluster_kernel(nt, S, v & 1, v & 2);
        e = allow_max_dynamic_smem(reinterpret_cast<const void *>(k), smem);
        if (e == cudaSuccess && csize > 8) e = cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    }
    return e;
}

int cluster_max_active(int csize, int nt, int S, size_t smem, int R)
{
    if (!cluster_threads_ok(nt, S)) return 0;
    // the variant with every term uses the most registers
    const ClusterKernel k = cluster_kernel(nt, S, true, true);
    if (allow_max_dynamic_smem(reinterpret_cast<const void *>(k), smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    if (csize > 8 && cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(csize * R, 1, 1);
    cfg.blockDim = dim3(nt, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = csize;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, k, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

cudaError_t launch_cluster(const ClusterArgs &a, int csize, int nt, int S, size_t smem, cudaStream_t st)
{
    if (!cluster_threads_ok(nt, S)) return cudaErrorInvalidValue;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(csize * a.R, 1, 1);
    cfg.blockDim = dim3(nt, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = csize;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, cluster_kernel(nt, S, a.has_b != 0, a.has_d != 0), a);
}

}  // namespace esp
