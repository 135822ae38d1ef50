// Launchers of the Monte Carlo kernels (esp_kernels.cu); host-side only.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "esp_device.cuh"

namespace esp {

struct EnergyArgsHost {
    const int32_t *nnb, *nbr;
    const float *J, *B, *Dx, *Dy, *Dz;
    const int32_t *perm;
    const float4 *si, *fld;
    const float *sx, *sy, *sz;
    double *scratch;          // [blocks][R][4]
    int32_t N, R, num_atoms;
};

struct FoldArgs {
    double *part;
    unsigned long long *part_rej;
    double *e_run, *m_run;
    unsigned long long *rej;  // [R slots][2]
    const int32_t *temp_of;
    int32_t R, nblocks, slots, block_threads, phase;
};

struct MeasureArgs {
    const double *e_run, *m_run;
    const int32_t *repl_at;
    double *data;             // [R][6]
    double *lsum, *binning;   // [R][nlev][2]
    const int32_t *levels;    // [nlev] (device)
    int32_t R, N, nlev, pt_quirk;
    long long step;           // 1-based measurement index
    double *series;           // [cap][R][2]: (E, |m|) per measurement, or null
    long long series_cap;
    const unsigned long long *ctr;   // device measurement counter added to step, or null
    // optional measurements, mcarlo.F90:553-568: bit 0 order parameter, bit 1
    // staggered magnetisation
    int32_t obs;
    const double *obs_rep;    // [R replicas] sum_i s_i.a_i, then [R replicas][3] sum_i c_i s_i
    double *obs_data;         // [R][6]: |OP|, OP^2, OP^4, |SM|, SM^2, SM^4 sums
    double *obs_lsum, *obs_bin;   // [R][nlev][2]: |OP|, |SM| binning
};

// Sums over the sites of every replica of s.a (order-parameter axis a of the
// site's atom) and c s (staggered coefficient c), for orderparam_get /
// staggered_get (get_quant.F90:366-422).
struct ObsArgs {
    const float *sx, *sy, *sz;
    const int32_t *perm;      // permuted index -> reference site
    const float4 *atom;       // [num_atoms]: axis (x, y, z), coefficient (w)
    double *scratch;          // [blocks][R][4]
    int32_t N, R, num_atoms;
};

// spincorr_get (get_quant.F90:495-540) per replica: for every bin b = (shell,
// species of the site, species of the neighbour) the sums over sites p of
// sum_{e in bin b} w_e (s_p . s_nb[e]) and of its magnitudes, with
// w = 1 / (shell_num_nbors_kind m_i m_j).  Entries of site p for bin b are
// off[b][p] .. off[b+1][p]-1 of the site-fastest lists nb / w.
struct ScArgs {
    const float *sx, *sy, *sz;
    const int32_t *off;       // [B+1][N]
    const int32_t *nb;        // [maxe][N], permuted neighbour index
    const float *w;           // [maxe][N]
    double *scratch;          // [npass][blocks][R][4], npass = ceil(B/2)
    double *out;              // [npass][R replicas][4]: bins 2k, 2k+1 (sum, sum |.|)
    double *acc;              // [R slots][B][3]: += sum, sum |.|, |sum|
    const int32_t *repl_at;
    int32_t N, R, B;
};

// mcarlo_structure_factor (get_quant.F90:649-717): F(q) = sum_i s_i e^{i q.r_i}
// per replica, q.r_i / 2 pi = nq . n_i + qf . f_i with n_i the site's integer
// lattice coordinates (phase in 32-bit fixed point, exact modulo one turn)
// and f_i its fractional remainder.
struct SfArgs {
    const float *sx, *sy, *sz;
    const int32_t *inv;       // reference site -> permuted index
    const int4 *site_n;       // [N]: integer lattice coordinates of the site
    const float4 *site_f;     // [N]: fractional remainder
    const uint4 *q_fix;       // [nq]: frac(qf_j) * 2^32, j = 1..3
    const float4 *q_frac;     // [nq]: qf_j (q in reciprocal-lattice units)
    const float4 *q_cart;     // [nq]: q (x, y, z), w = 1 if q is exactly zero
    float *fq;                // [R replicas][nq][6]: Re/Im of F_x, F_y, F_z
    double *acc;              // [R slots][nq][3]: += |F_perp|^2, |F_perp|^2 - NSF^2, NSF^2
    unsigned long long *count;   // number of structure-factor measurements
    const int32_t *repl_at;
    double px, py, pz, pnorm;    // sfactor_polar and its length
    int32_t N, R, nq, every;     // measure when step % every == 0
    long long step;              // 1-based measurement index (relative under capture)
    const unsigned long long *ctr;   // device measurement counter added to step, or null
};

struct PmArgs {
    const float *sx, *sy, *sz;
    const int32_t *inv;       // reference site -> permuted index
    const int32_t *temp_of;
    unsigned long long *counts;  // [R slots][nf]
    int32_t R, ncell, num_atoms, nf, use_shared, rt;
    double m_min, m_max;
    int32_t count_m;          // bin |sum s| (P(M)) into counts
    int32_t obs;              // bit 0: P(OP), bit 1: P(SM) into obs_counts
    const float4 *obs_atom;   // [num_atoms]: axis (x, y, z), coefficient (w)
    unsigned long long *obs_counts;  // [R slots][2][nf]
};

struct PtSwapArgs {
    int32_t *repl_at, *temp_of;
    const double *e_run, *inv_t;
    long long *num_swaps;     // [R][2]
    int32_t R, start0;
    uint32_t key0, key1, idx_lo, idx_hi;
    int32_t group;            // temperatures per independent lattice (R for one lattice)
    // device counters [sweep, swap, measurement, unit] or null: the swap index
    // adds ctr[1]; the start pair follows the parity of unit ctr[3] + unit_off
    const unsigned long long *ctr;
    int32_t unit_off;
};

int sweep_blocks(long long max_items, int R, int max_blocks);
cudaError_t launch_sweep(const SweepArgs &a, bool hb, bool hd, int blocks, cudaStream_t st);
cudaError_t launch_fold(const FoldArgs &a, cudaStream_t st);
int energy_blocks(int N, int R, int max_blocks);
cudaError_t launch_energy(const EnergyArgsHost &h, double *out_e, double *out_m, int blocks, cudaStream_t st);
cudaError_t launch_local_terms(const EnergyArgsHost &h, float *g, float *q, cudaStream_t st);
cudaError_t launch_measure(const MeasureArgs &a, cudaStream_t st);
// out_op[r] = sum_i s_i.a_i, out_sm[3r..3r+2] = sum_i c_i s_i; scratch holds
// blocks x R x 4 doubles (the energy scratch serves)
cudaError_t launch_obs(const ObsArgs &a, double *out_op, double *out_sm, int blocks, cudaStream_t st);
cudaError_t launch_pm(const PmArgs &a, int max_blocks, cudaStream_t st);
// one spincorr_get measurement of every replica, accumulated per slot
cudaError_t launch_spincorr(const ScArgs &a, int blocks, cudaStream_t st);
// one structure-factor measurement of every replica if step % every == 0
cudaError_t launch_sfactor(const SfArgs &a, cudaStream_t st);
cudaError_t launch_pt_swap(const PtSwapArgs &a, cudaStream_t st);
// ctr[i] += d[i] for the four run counters
cudaError_t launch_bump(unsigned long long *ctr, const unsigned long long d[4], cudaStream_t st);
// spin_matrix(3, N, slots t0 .. t0+nt-1) staged on the device <-> the state
cudaError_t launch_spins_in(const double *stage, const int32_t *inv, const int32_t *repl_at, float *sx, float *sy,
                            float *sz, int N, int R, int t0, int nt, cudaStream_t st);
cudaError_t launch_spins_out(double *stage, const int32_t *inv, const int32_t *repl_at, const float *sx,
                             const float *sy, const float *sz, int N, int R, int t0, int nt, cudaStream_t st);
cudaError_t launch_init_spins(const int32_t *perm, const float *mag, float *sx, float *sy, float *sz,
                              int N, int R, int kind, uint64_t seed, cudaStream_t st);

}  // namespace esp
