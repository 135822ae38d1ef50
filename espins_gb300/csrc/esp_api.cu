// C ABI of libespins_gpu.so (declared in include/espins_gpu.h): the handle,
// device memory, and the schedules of mcarlo (ESpinS src/mcarlo.F90:463-733)
// and pt_mcarlo (src/pt.F90:504-1024) driven from the host.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/espins_gpu.h"
#include "esp_cluster.h"
#include "esp_kernels.h"
#include "esp_learned.h"
#include "esp_lp_tc.h"
#include "esp_tile.h"
#include "esp_tables.h"
#include "esp_errors.h"

using namespace esp;

struct RunState {
    bool active = false;
    esp_schedule s{};
    std::vector<int32_t> levels;
    int nlev = 0;
    int64_t total_units = 0, units_done = 0, meas_done = 0;
    long long const_hits = 0;
    int64_t steps_tot[2] = {0, 0};
    std::vector<double> e_init;
};

struct esp_handle {
    RunState run;
    std::string err;
    int N = 0, R = 0, na = 0, L[3] = {0, 0, 0};
    bool open = false;
    cudaStream_t own = nullptr, st = nullptr;
    int device = 0, num_sms = 0, max_blocks = 0;
    long long launches = 0;
    bool have_tables = false, have_temps = false;
    int64_t next_sweep = 0, next_swap = 0;
    // tables
    PrepOutput prep;
    bool hsi = false, hfld = false;
    int32_t *d_nnb = nullptr, *d_nbr = nullptr, *d_perm = nullptr, *d_inv = nullptr;
    float *d_J = nullptr, *d_B = nullptr, *d_Dx = nullptr, *d_Dy = nullptr, *d_Dz = nullptr, *d_mag = nullptr;
    float4 *d_si = nullptr, *d_fld = nullptr;
    // state
    float *d_sx = nullptr, *d_sy = nullptr, *d_sz = nullptr;
    int32_t *d_temp_of = nullptr, *d_repl_at = nullptr;
    float *d_beta = nullptr;
    double *d_inv_t = nullptr;
    double *d_e_run = nullptr, *d_m_run = nullptr;
    unsigned long long *d_rej = nullptr;
    double *d_scratch = nullptr;
    int e_blocks = 0;
    // per-block partial sums of the sweeps (see add_block_slots / k_fold)
    double *d_part = nullptr;
    unsigned long long *d_part_rej = nullptr;
    int sweep_grid = 0, slots = 0;
    int part_blocks = 0;            // 256-thread blocks with partial slots (>= sweep_grid)
    int pending_phase = 0;
    long long pending_sweeps = 0;
    // cluster-resident path (translation-invariant lattices)
    int kernel_choice = 0;          // 0 auto, 1 ELL, 2 cluster
    bool cluster_ok = false;
    int csize = 0, pz = 0, cthreads = 512, csites = 1;
    int cl_nA = 0;                  // ranks with pz planes; the others hold pz - 2
    // Which copy of the spins is current: the spin arrays (element (p, r) at
    // p*R + r) and/or the cluster path's slab copy.  The cluster kernel leaves
    // the state in the slabs; the arrays are brought up to date (one
    // transpose) only when something else reads them, and the slabs only when
    // the cluster kernel runs after something wrote the arrays.  At least one
    // of the two always holds the state.
    bool arrays_ok = true, slab_ok = false;
    size_t cluster_smem = 0;
    int cl_maxst = 0;
    size_t cl_sbytes = 0;
    // tiled path (translation-invariant lattices with nearest-cell stencils)
    bool tile_ok = false;
    int tile_T = 0, tile_G = 0, tile_nt[3] = {0, 0, 0}, ntiles = 0;
    int tile_variant = 0;           // 0 one CTA per tile; pipelined persistent: 1 one CTA per SM, 2 two
    int tile_blocks = 0;            // persistent grid of the pipelined variants
    size_t tile_smem = 0;
    int4 *d_tile_offs = nullptr;
    ClusterNbr *d_tile_cpl = nullptr;
    int tile_maxst = 0, tile_nbd8[kMaxClusterAtoms] = {}, tile_nall8[kMaxClusterAtoms] = {};
    int tile_nbd2[kMaxClusterAtoms] = {}, tile_nall4[kMaxClusterAtoms] = {};
    double *d_tile_part = nullptr;
    unsigned long long *d_tile_rej = nullptr;
    long long tile_pending = 0;
    double *d_series = nullptr;
    long long series_cap = 0;
    unsigned char *d_stencil_blob = nullptr;
    uint32_t *d_nbidx = nullptr;
    int stencil_words = 0;
    double *d_tmp_e = nullptr, *d_tmp_m = nullptr;
    // accumulators
    double *d_data = nullptr, *d_lsum = nullptr, *d_bin = nullptr;
    int32_t *d_levels = nullptr;
    int nlev_alloc = 0;
    unsigned long long *d_pm = nullptr;
    long long *d_swaps = nullptr;
    // optional measurements (esp_set_observables): bit 0 order parameter,
    // bit 1 staggered magnetisation
    int obs = 0;
    float4 *d_obs_atom = nullptr;           // [na]: axis (x, y, z), coefficient (w)
    double *d_obs_rep = nullptr;            // [R replicas] sum s.a, then [R replicas][3] sum c s
    double *d_obs_data = nullptr;           // [R slots][6]
    double *d_obs_lsum = nullptr, *d_obs_bin = nullptr;   // [R slots][nlev_alloc][2]
    unsigned long long *d_obs_pm = nullptr; // [R slots][2][nf]
    // spin correlations (esp_set_spin_correlation): B bins = shells x
    // species x species, per-site entry lists grouped by bin
    int sc_B = 0, sc_S = 0, sc_nsp = 0, sc_blocks = 0;
    int32_t *d_sc_off = nullptr, *d_sc_nb = nullptr;
    float *d_sc_w = nullptr;
    double *d_sc_scratch = nullptr, *d_sc_out = nullptr, *d_sc_acc = nullptr;
    std::vector<double> mag_host;   // mag_moments_matrix, reference order
    // staging of spin_matrix blocks for esp_set_spins / esp_get_spins, and a
    // pinned host copy that esp_get_spins reads back through (a copy straight
    // into the caller's pages would fault them in inside the transfer)
    double *d_stage = nullptr, *h_stage = nullptr;
    float *d_slab = nullptr;   // spins in the cluster path's slab layout during its launches
    int stage_slots = 0;
    // the device reads / writes pageable host memory through the host's page
    // tables (a coherent CPU-GPU link): the spin transfers can skip the
    // staging.  host_transfer: bit 0 esp_set_spins reads the caller's array,
    // bit 1 esp_get_spins writes it, -1 the default
    bool host_direct_ok = false;
    int host_transfer = -1;
    cudaEvent_t stage_ev[2] = {nullptr, nullptr};   // a staging half's copy has finished
    // structure factor (esp_set_structure_factor)
    int sf_nq = 0, sf_every = 1;
    double sf_p[3] = {1.0, 0.0, 0.0}, sf_pnorm = 1.0;
    int4 *d_sf_n = nullptr;
    float4 *d_sf_f = nullptr, *d_sf_qf = nullptr, *d_sf_qc = nullptr;
    uint4 *d_sf_qfix = nullptr;
    float *d_sf_fq = nullptr;
    double *d_sf_acc = nullptr;
    unsigned long long *d_sf_count = nullptr;
    std::vector<double> tems;
    int nf = 2;
    double m_min = 0, m_max = 0;
    // learned proposal: network (fp32 master + Adam moments + bf16 copies),
    // training set, mini-batch buffers
    int proposal = 0;               // 0 plain Metropolis, 1 learned
    int lp_engine = 0;              // network on 0: mma.sync (warp tiles), 1: tcgen05 (128-row tiles)
    int *d_tc_err = nullptr;        // set by a tensor-core completion wait that gave up
    int tc_force_timeout = 0;       // test hook: tcgen05 waits report a give-up (esp_lp_force_tc_timeout)
    float *d_lp_gwork = nullptr;    // partial tiles of the tcgen05 training GEMMs split along K
    // partial sums of the tcgen05 learned sweep (128-thread blocks)
    int tc_grid = 0, tc_slots = 0;
    double *d_tc_part = nullptr;
    unsigned long long *d_tc_part_rej = nullptr;
    long long tc_pending = 0;
    bool lp_weights = false;
    int lp_grid = 0;
    float *d_lp_p = nullptr, *d_lp_g = nullptr, *d_lp_m = nullptr, *d_lp_v = nullptr;
    __nv_bfloat16 *d_lp_w1 = nullptr, *d_lp_w2 = nullptr, *d_lp_w3 = nullptr;
    float4 *d_lp_axis = nullptr;
    long long lp_adam_t = 0;
    __nv_bfloat16 *d_lp_x = nullptr;
    float *d_lp_t = nullptr;
    long long lp_cap = 0, lp_n = 0;
    int lp_bcap = 0;
    __nv_bfloat16 *d_lp_xb = nullptr, *d_lp_h1 = nullptr, *d_lp_h2 = nullptr, *d_lp_do = nullptr,
                  *d_lp_dz2 = nullptr, *d_lp_dz1 = nullptr;
    float *d_lp_tb = nullptr, *d_lp_o = nullptr;
    double *d_lp_loss = nullptr;
    long long lp_loss_cap = 0;
    // PT: temperatures per independent lattice (0: all R are one lattice)
    int pt_group = 0;
    // run counters on the device [sweep, swap, measurement, unit], used by
    // kernels launched inside a captured graph: their arguments hold values
    // relative to the counters at capture time and every replay advances
    // the counters (k_bump) instead of repeating the same random numbers
    unsigned long long *d_ctr = nullptr;
    unsigned long long ctr_shadow[4] = {0, 0, 0, 0};   // what d_ctr holds
    bool ctr_valid = false;
    bool capturing = false;
    int64_t cap_base[4] = {0, 0, 0, 0};
};

namespace {

// Message of the last failure that has no handle to hold it (esp_create and
// calls without a handle); a fixed buffer, so recording it allocates nothing.
char g_global_err[512] = "";

#define CK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) {                                                                   \
            h->err = std::string(#call) + ": " + cudaGetErrorString(e_);                           \
            return ESP_ECUDA;                                                                      \
        }                                                                                          \
    } while (0)

template <class T>
cudaError_t dalloc(T **p, size_t n)
{
    if (n == 0) n = 1;
    return cudaMalloc((void **)p, n * sizeof(T));
}

template <class T>
void dfree(T *&p)
{
    if (p) cudaFree((void *)p);
    p = nullptr;
}

void free_tables(esp_handle *h)
{
    dfree(h->d_nnb); dfree(h->d_nbr); dfree(h->d_perm); dfree(h->d_inv);
    dfree(h->d_J); dfree(h->d_B); dfree(h->d_Dx); dfree(h->d_Dy); dfree(h->d_Dz); dfree(h->d_mag);
    dfree(h->d_si); dfree(h->d_fld); dfree(h->d_scratch); dfree(h->d_part); dfree(h->d_part_rej);
    dfree(h->d_tc_part); dfree(h->d_tc_part_rej);
    dfree(h->d_stencil_blob); dfree(h->d_nbidx); dfree(h->d_lp_axis); dfree(h->d_slab);
    dfree(h->d_tile_offs); dfree(h->d_tile_cpl); dfree(h->d_tile_part); dfree(h->d_tile_rej);
    h->cluster_ok = false;
    h->tile_ok = false;
}

void free_obs(esp_handle *h)
{
    dfree(h->d_obs_atom); dfree(h->d_obs_rep); dfree(h->d_obs_data); dfree(h->d_obs_pm);
    h->obs = 0;
}

void free_sf(esp_handle *h)
{
    dfree(h->d_sf_n); dfree(h->d_sf_f); dfree(h->d_sf_qf); dfree(h->d_sf_qc); dfree(h->d_sf_qfix);
    dfree(h->d_sf_fq); dfree(h->d_sf_acc); dfree(h->d_sf_count);
    h->sf_nq = 0;
}

void free_sc(esp_handle *h)
{
    dfree(h->d_sc_off); dfree(h->d_sc_nb); dfree(h->d_sc_w);
    dfree(h->d_sc_scratch); dfree(h->d_sc_out); dfree(h->d_sc_acc);
    h->sc_B = h->sc_S = h->sc_nsp = 0;
}

void free_lp_batch(esp_handle *h)
{
    dfree(h->d_lp_xb); dfree(h->d_lp_h1); dfree(h->d_lp_h2); dfree(h->d_lp_do); dfree(h->d_lp_dz2);
    dfree(h->d_lp_dz1); dfree(h->d_lp_tb); dfree(h->d_lp_o);
    h->lp_bcap = 0;
}

void free_all(esp_handle *h)
{
    free_tables(h);
    dfree(h->d_sx); dfree(h->d_sy); dfree(h->d_sz);
    dfree(h->d_temp_of); dfree(h->d_repl_at); dfree(h->d_beta); dfree(h->d_inv_t);
    dfree(h->d_e_run); dfree(h->d_m_run); dfree(h->d_rej); dfree(h->d_tmp_e); dfree(h->d_tmp_m);
    dfree(h->d_data); dfree(h->d_lsum); dfree(h->d_bin); dfree(h->d_levels); dfree(h->d_pm); dfree(h->d_swaps);
    dfree(h->d_obs_lsum); dfree(h->d_obs_bin);
    free_obs(h);
    free_sc(h);
    free_sf(h);
    dfree(h->d_stage);
    if (h->h_stage) cudaFreeHost(h->h_stage);
    h->h_stage = nullptr;
    h->stage_slots = 0;
    for (cudaEvent_t &ev : h->stage_ev) {
        if (ev) cudaEventDestroy(ev);
        ev = nullptr;
    }
    dfree(h->d_series);
    free_lp_batch(h);
    dfree(h->d_lp_p); dfree(h->d_lp_g); dfree(h->d_lp_m); dfree(h->d_lp_v);
    dfree(h->d_lp_w1); dfree(h->d_lp_w2); dfree(h->d_lp_w3);
    dfree(h->d_lp_x); dfree(h->d_lp_t); dfree(h->d_lp_loss);
    dfree(h->d_ctr);
    dfree(h->d_tc_err);
    dfree(h->d_lp_gwork);
}

SweepArgs sweep_args(esp_handle *h, int c, int64_t sweep, const esp_sweep_opts *o)
{
    SweepArgs a;
    a.nnb = h->d_nnb; a.nbr = h->d_nbr; a.J = h->d_J; a.B = h->d_B;
    a.Dx = h->d_Dx; a.Dy = h->d_Dy; a.Dz = h->d_Dz;
    a.perm = h->d_perm; a.mag = h->d_mag; a.si = h->hsi ? h->d_si : nullptr; a.fld = h->hfld ? h->d_fld : nullptr;
    a.sx = h->d_sx; a.sy = h->d_sy; a.sz = h->d_sz;
    a.temp_of = h->d_temp_of; a.beta = h->d_beta;
    a.part = h->d_part; a.part_rej = h->d_part_rej; a.slots = h->slots;
    a.N = h->N; a.R = h->R; a.num_atoms = h->na;
    a.off_c = h->prep.off[c]; a.n_c = h->prep.off[c + 1] - h->prep.off[c];
    a.mode = o->mcarlo_mode ? 1 : 0; a.tilt = (float)o->tilt_angles_max;
    a.key0 = (uint32_t)o->seed; a.key1 = (uint32_t)(o->seed >> 32);
    a.ctr = nullptr;
    if (h->capturing) {
        sweep -= h->cap_base[0];
        a.ctr = h->d_ctr;
    }
    a.sw_lo = (uint32_t)sweep; a.sw_hi = (uint32_t)((uint64_t)sweep >> 32);
    return a;
}

EnergyArgsHost energy_args(esp_handle *h)
{
    EnergyArgsHost a;
    a.nnb = h->d_nnb; a.nbr = h->d_nbr; a.J = h->d_J; a.B = h->d_B;
    a.Dx = h->d_Dx; a.Dy = h->d_Dy; a.Dz = h->d_Dz;
    a.perm = h->d_perm; a.si = h->hsi ? h->d_si : nullptr; a.fld = h->hfld ? h->d_fld : nullptr;
    a.sx = h->d_sx; a.sy = h->d_sy; a.sz = h->d_sz;
    a.scratch = h->d_scratch; a.N = h->N; a.R = h->R; a.num_atoms = h->na;
    return a;
}

int require(esp_handle *h, bool tables, bool temps)
{
    if (!h) return ESP_EINVAL;
    if (tables && !h->have_tables) { h->err = "tables not uploaded (esp_upload_tables)"; return ESP_ESTATE; }
    if (temps && !h->have_temps) { h->err = "temperatures not set (esp_set_temperatures)"; return ESP_ESTATE; }
    return ESP_OK;
}

// Adds the sweeps' per-block partial sums to the running energies,
// magnetisations and rejected counters (k_fold), in block order.
int fold(esp_handle *h)
{
    if (h->tc_pending > 0) {
        FoldArgs f;
        f.part = h->d_tc_part; f.part_rej = h->d_tc_part_rej; f.e_run = h->d_e_run; f.m_run = h->d_m_run;
        f.rej = h->d_rej; f.temp_of = h->d_temp_of; f.R = h->R; f.nblocks = h->tc_grid; f.slots = h->tc_slots;
        f.block_threads = 128; f.phase = h->pending_phase;
        CK(launch_fold(f, h->st));
        h->launches++;
        h->tc_pending = 0;
    }
    if (h->tile_pending > 0) {
        TileFoldArgs t;
        t.part = h->d_tile_part; t.part_rej = h->d_tile_rej; t.e_run = h->d_e_run; t.m_run = h->d_m_run;
        t.rej = h->d_rej; t.temp_of = h->d_temp_of; t.R = h->R; t.ntiles = h->ntiles; t.phase = h->pending_phase;
        CK(launch_tile_fold(t, h->st));
        h->launches += 2;
        h->tile_pending = 0;
    }
    if (h->pending_sweeps == 0) return ESP_OK;
    FoldArgs f;
    f.part = h->d_part; f.part_rej = h->d_part_rej; f.e_run = h->d_e_run; f.m_run = h->d_m_run;
    f.rej = h->d_rej; f.temp_of = h->d_temp_of; f.R = h->R; f.nblocks = h->part_blocks; f.slots = h->slots;
    f.block_threads = 256; f.phase = h->pending_phase;
    CK(launch_fold(f, h->st));
    h->launches++;
    h->pending_sweeps = 0;
    return ESP_OK;
}

bool use_cluster(const esp_handle *h)
{
    return h->cluster_ok && (h->kernel_choice == 0 || h->kernel_choice == 2) && h->proposal == 0;
}

// the tiled kernel: when chosen, or by default where no cluster fits
bool use_tile(const esp_handle *h)
{
    return h->tile_ok && h->proposal == 0 &&
           (h->kernel_choice == 4 || (h->kernel_choice == 0 && !h->cluster_ok));
}

// n sweeps of eight tile-parity launches each
int arrays_current(esp_handle *h);
void arrays_written(esp_handle *h);

int tile_sweeps(esp_handle *h, int64_t n, int64_t first, const esp_sweep_opts *o)
{
    int rc0 = arrays_current(h);
    if (rc0) return rc0;
    arrays_written(h);
    const int phase = o->phase ? 1 : 0;
    if (phase != h->pending_phase) {
        int rc = fold(h);
        if (rc) return rc;
        h->pending_phase = phase;
    }
    TileArgs a;
    a.stencil = reinterpret_cast<const ClusterStencil *>(h->d_stencil_blob);
    a.offs = h->d_tile_offs;
    a.cpl = h->d_tile_cpl;
    a.maxst = h->tile_maxst;
    for (int at = 0; at < kMaxClusterAtoms; ++at) {
        a.nbd8[at] = h->tile_nbd8[at];
        a.nall8[at] = h->tile_nall8[at];
        a.nbd2[at] = h->tile_nbd2[at];
        a.nall4[at] = h->tile_nall4[at];
    }
    a.Lx = h->L[0]; a.Ly = h->L[1]; a.Lz = h->L[2]; a.na = h->na; a.N = h->N; a.R = h->R;
    a.T = h->tile_T; a.G = h->tile_G;
    a.ntx = h->tile_nt[0]; a.nty = h->tile_nt[1]; a.ntz = h->tile_nt[2];
    a.has_b = h->prep.has_b; a.has_d = h->prep.has_d; a.has_si = h->hsi; a.has_f = h->hfld;
    a.sx = h->d_sx; a.sy = h->d_sy; a.sz = h->d_sz; a.inv = h->d_inv;
    a.temp_of = h->d_temp_of; a.beta = h->d_beta;
    a.part = h->d_tile_part; a.part_rej = h->d_tile_rej;
    a.key0 = (uint32_t)o->seed; a.key1 = (uint32_t)(o->seed >> 32);
    a.mode = o->mcarlo_mode ? 1 : 0; a.tilt = (float)o->tilt_angles_max;
    a.ctr = h->capturing ? h->d_ctr : nullptr;
    for (int64_t w = 0; w < n; ++w) {
        a.sweep = (unsigned long long)(first + w - (h->capturing ? h->cap_base[0] : 0));
        for (int ph = 0; ph < 8; ++ph) {
            a.phase = ph;
            if (h->tile_variant) CK(launch_tile_p(a, h->tile_smem, h->tile_blocks, 3 - h->tile_variant, h->st));
            else CK(launch_tile(a, h->tile_smem, h->st));
            h->launches++;
        }
        h->tile_pending++;
    }
    return ESP_OK;
}

// One launch of the cluster-resident kernel: n_meas units of steps_measure
// sweeps starting at global sweep `first`, each unit followed by a
// measurement when `measure` is set.
SlabArgs slab_args(const esp_handle *h)
{
    SlabArgs sa;
    sa.sx = h->d_sx; sa.sy = h->d_sy; sa.sz = h->d_sz; sa.slab = h->d_slab; sa.inv = h->d_inv;
    sa.Lx = h->L[0]; sa.Ly = h->L[1]; sa.na = h->na; sa.R = h->R; sa.pz = h->pz; sa.nA = h->cl_nA;
    sa.cs = h->csize; sa.N = h->N;
    sa.n_local = (h->L[0] / 2) * (h->L[1] / 2) * (h->pz / 2) * 8 * h->na;
    sa.fd_pc = make_fastdiv((uint32_t)((h->L[0] / 2) * (h->L[1] / 2) * (h->pz / 2)));
    sa.fd_pc2 = make_fastdiv((uint32_t)std::max(1, (h->L[0] / 2) * (h->L[1] / 2) * (h->pz / 2 - 1)));
    sa.fd_hx = make_fastdiv((uint32_t)(h->L[0] / 2));
    sa.fd_hy = make_fastdiv((uint32_t)(h->L[1] / 2));
    return sa;
}

// Slabs of at least 4096 sites are staged contiguously (two transposes);
// smaller ones are gathered and scattered by the cluster kernel itself.
bool cluster_staged(const esp_handle *h)
{
    return h->cluster_ok && h->csize > 0 && h->N / h->csize >= 4096;
}

// Bring the spin arrays up to date before a kernel reads them.
int arrays_current(esp_handle *h)
{
    if (h->arrays_ok) return ESP_OK;
    CK(launch_from_slabs(slab_args(h), h->st));
    h->launches++;
    h->arrays_ok = true;
    return ESP_OK;
}

// A kernel wrote the spin arrays: the slab copy is stale.
void arrays_written(esp_handle *h)
{
    h->arrays_ok = true;
    h->slab_ok = false;
}

// Bring the slab copy up to date before the cluster kernel works on it.
int slab_current(esp_handle *h)
{
    if (h->slab_ok) return ESP_OK;
    CK(launch_to_slabs(slab_args(h), h->st));
    h->launches++;
    h->slab_ok = true;
    return ESP_OK;
}

int cluster_run(esp_handle *h, int64_t n_meas, int steps_measure, int64_t first, int measure, long long meas_base,
                const esp_sweep_opts *o, int phase, int nlev, bool pt_quirk)
{
    int rc = fold(h);
    if (rc) return rc;
    ClusterArgs a;
    a.stencil = reinterpret_cast<const ClusterStencil *>(h->d_stencil_blob);
    a.stencil_words = h->stencil_words;
    a.nbidx = h->d_nbidx;
    a.Lx = h->L[0]; a.Ly = h->L[1]; a.Lz = h->L[2]; a.na = h->na; a.N = h->N; a.R = h->R;
    a.nclass = 8 * h->na; a.pz = h->pz; a.nA = h->cl_nA;
    a.has_b = h->prep.has_b; a.has_d = h->prep.has_d; a.has_si = h->hsi; a.has_f = h->hfld;
    const bool staged = cluster_staged(h);
    a.slab = staged ? h->d_slab : nullptr;
    a.sx = h->d_sx; a.sy = h->d_sy; a.sz = h->d_sz; a.inv = h->d_inv;
    a.temp_of = h->d_temp_of; a.beta = h->d_beta; a.e_run = h->d_e_run; a.m_run = h->d_m_run; a.rej = h->d_rej;
    a.phase = phase;
    a.measure = measure; a.n_meas = (int)n_meas; a.steps_measure = steps_measure; a.meas_base = meas_base;
    a.data = h->d_data; a.lsum = h->d_lsum; a.binning = h->d_bin; a.levels = h->d_levels;
    a.nlev = nlev; a.pt_quirk = pt_quirk ? 1 : 0;
    a.pm_counts = h->d_pm; a.nf = h->nf; a.m_min = h->m_min; a.m_max = h->m_max;
    a.series = h->d_series; a.series_cap = h->series_cap;
    a.ctr = nullptr;
    if (h->capturing) {
        first -= h->cap_base[0];
        a.meas_base -= h->cap_base[2];
        a.ctr = h->d_ctr;
    }
    a.sweep_base = (unsigned long long)first;
    a.fd_pc = make_fastdiv((uint32_t)((h->L[0] / 2) * (h->L[1] / 2) * (h->pz / 2)));
    a.fd_pc2 = make_fastdiv((uint32_t)std::max(1, (h->L[0] / 2) * (h->L[1] / 2) * (h->pz / 2 - 1)));
    a.fd_hx = make_fastdiv((uint32_t)(h->L[0] / 2));
    a.fd_hy = make_fastdiv((uint32_t)(h->L[1] / 2));
    a.rn_inv = 1.0 / (double)h->N;
    a.key0 = (uint32_t)o->seed; a.key1 = (uint32_t)(o->seed >> 32);
    a.mode = o->mcarlo_mode ? 1 : 0; a.tilt = (float)o->tilt_angles_max;
    a.obs = measure ? h->obs : 0;
    a.obs_atom = h->d_obs_atom; a.obs_data = h->d_obs_data; a.obs_lsum = h->d_obs_lsum; a.obs_bin = h->d_obs_bin;
    a.obs_pm = h->d_obs_pm;
    // a staged slab stays the state after the launch (the arrays are brought
    // back by a transpose when something reads them); an unstaged launch
    // reads and writes the arrays themselves
    if (staged) {
        if ((rc = slab_current(h))) return rc;
    } else if ((rc = arrays_current(h))) {
        return rc;
    }
    CK(launch_cluster(a, h->csize, h->cthreads, h->csites, h->cluster_smem, h->st));
    h->launches++;
    if (staged) h->arrays_ok = false;
    else arrays_written(h);
    return ESP_OK;
}

// plain sweeps on the cluster path, in launches of at most kChunk sweeps
constexpr int64_t kChunk = 1000;

int cluster_sweeps(esp_handle *h, int64_t n, int64_t first, const esp_sweep_opts *o)
{
    for (int64_t done = 0; done < n; done += kChunk) {
        const int64_t k = std::min(kChunk, n - done);
        int rc = cluster_run(h, k, 1, first + done, 0, 0, o, o->phase ? 1 : 0, 0, false);
        if (rc) return rc;
    }
    return ESP_OK;
}

int do_sweep_colour(esp_handle *h, int c, int64_t sweep, const esp_sweep_opts *o)
{
    int rc0 = arrays_current(h);
    if (rc0) return rc0;
    arrays_written(h);
    const int phase = o->phase ? 1 : 0;
    if (phase != h->pending_phase) {
        int rc = fold(h);
        if (rc) return rc;
        h->pending_phase = phase;
    }
    SweepArgs a = sweep_args(h, c, sweep, o);
    if (a.n_c == 0) return ESP_OK;
    if (h->proposal == 1) {
        LpSweepArgs la;
        la.s = a;
        la.w.w1 = h->d_lp_w1; la.w.w2 = h->d_lp_w2; la.w.w3 = h->d_lp_w3;
        la.w.b1 = h->d_lp_p + kPadB1; la.w.b2 = h->d_lp_p + kPadB2; la.w.b3 = h->d_lp_p + kPadB3;
        la.axis = h->hsi ? h->d_lp_axis : nullptr;
        la.tc_force_timeout = h->tc_force_timeout;
        if (h->lp_engine == 1) {
            // d_tc_err exists: esp_lp_set_engine allocates it (no allocation here,
            // this may run inside a graph capture)
            CK(launch_sweep_lp_tc(la, h->prep.has_b, h->prep.has_d, h->tc_grid, h->d_tc_part, h->d_tc_part_rej,
                                  h->tc_slots, h->d_tc_err, h->st));
            h->launches++;
            h->tc_pending++;
            return ESP_OK;
        }
        CK(launch_sweep_lp(la, h->prep.has_b, h->prep.has_d, h->lp_grid, h->st));
    } else {
        CK(launch_sweep(a, h->prep.has_b, h->prep.has_d, h->sweep_grid, h->st));
    }
    h->launches++;
    h->pending_sweeps++;
    return ESP_OK;
}

int do_sweeps(esp_handle *h, int64_t n, int64_t first, const esp_sweep_opts *o)
{
    if (use_cluster(h)) return cluster_sweeps(h, n, first, o);
    if (use_tile(h)) return tile_sweeps(h, n, first, o);
    for (int64_t w = 0; w < n; ++w) {
        for (int c = 0; c < h->prep.num_colours; ++c) {
            int rc = do_sweep_colour(h, c, first + w, o);
            if (rc) return rc;
        }
        // keep the partial counters far from overflow on long warm-ups
        if (h->pending_sweeps >= 4096 * (long long)h->prep.num_colours) {
            int rc = fold(h);
            if (rc) return rc;
        }
    }
    return ESP_OK;
}

// energy by replica into d_tmp_e / d_tmp_m
int do_energy(esp_handle *h)
{
    int rc = arrays_current(h);
    if (rc) return rc;
    CK(launch_energy(energy_args(h), h->d_tmp_e, h->d_tmp_m, h->e_blocks, h->st));
    h->launches += 2;
    return ESP_OK;
}

int reset_running(esp_handle *h)
{
    // keep the rejected counts of pending sweeps, then overwrite the running
    // energies and magnetisations with direct ones
    int rc = fold(h);
    if (rc) return rc;
    if ((rc = do_energy(h))) return rc;
    CK(cudaMemcpyAsync(h->d_e_run, h->d_tmp_e, sizeof(double) * h->R, cudaMemcpyDeviceToDevice, h->st));
    CK(cudaMemcpyAsync(h->d_m_run, h->d_tmp_m, sizeof(double) * 3 * h->R, cudaMemcpyDeviceToDevice, h->st));
    return ESP_OK;
}

int identity_labels(esp_handle *h)
{
    std::vector<int32_t> id(h->R);
    for (int r = 0; r < h->R; ++r) id[r] = r;
    CK(cudaMemcpyAsync(h->d_temp_of, id.data(), sizeof(int32_t) * h->R, cudaMemcpyHostToDevice, h->st));
    CK(cudaMemcpyAsync(h->d_repl_at, id.data(), sizeof(int32_t) * h->R, cudaMemcpyHostToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
    return ESP_OK;
}

int get_repl_at(esp_handle *h, std::vector<int32_t> &ra)
{
    ra.resize(h->R);
    CK(cudaMemcpyAsync(ra.data(), h->d_repl_at, sizeof(int32_t) * h->R, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    return ESP_OK;
}

int by_slot(esp_handle *h, const double *d_by_rep, int width, double *out)
{
    std::vector<int32_t> ra;
    int rc = get_repl_at(h, ra);
    if (rc) return rc;
    std::vector<double> v((size_t)h->R * width);
    CK(cudaMemcpyAsync(v.data(), d_by_rep, sizeof(double) * width * h->R, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    for (int t = 0; t < h->R; ++t)
        for (int c = 0; c < width; ++c) out[(size_t)t * width + c] = v[(size_t)ra[t] * width + c];
    return ESP_OK;
}

// One spincorr_get measurement of every replica, accumulated per slot.
int spincorr_measure(esp_handle *h)
{
    int rc0 = arrays_current(h);
    if (rc0) return rc0;
    ScArgs a;
    a.sx = h->d_sx; a.sy = h->d_sy; a.sz = h->d_sz;
    a.off = h->d_sc_off; a.nb = h->d_sc_nb; a.w = h->d_sc_w;
    a.scratch = h->d_sc_scratch; a.out = h->d_sc_out; a.acc = h->d_sc_acc; a.repl_at = h->d_repl_at;
    a.N = h->N; a.R = h->R; a.B = h->sc_B;
    CK(launch_spincorr(a, h->sc_blocks, h->st));
    h->launches += 3;
    return ESP_OK;
}

// The structure factor after measurement `step` (1-based) when step is a
// multiple of sfactor_steps_measure; inside a graph capture the kernels test
// the step against the device measurement counter instead.
int sfactor_measure(esp_handle *h, long long step)
{
    int rc0 = arrays_current(h);
    if (rc0) return rc0;
    SfArgs a;
    a.sx = h->d_sx; a.sy = h->d_sy; a.sz = h->d_sz; a.inv = h->d_inv;
    a.site_n = h->d_sf_n; a.site_f = h->d_sf_f; a.q_fix = h->d_sf_qfix; a.q_frac = h->d_sf_qf; a.q_cart = h->d_sf_qc;
    a.fq = h->d_sf_fq; a.acc = h->d_sf_acc; a.count = h->d_sf_count; a.repl_at = h->d_repl_at;
    a.px = h->sf_p[0]; a.py = h->sf_p[1]; a.pz = h->sf_p[2]; a.pnorm = h->sf_pnorm;
    a.N = h->N; a.R = h->R; a.nq = h->sf_nq; a.every = h->sf_every;
    a.step = step; a.ctr = nullptr;
    if (h->capturing) {
        a.step -= h->cap_base[2];
        a.ctr = h->d_ctr + 2;
    } else if (step % h->sf_every != 0) {
        return ESP_OK;
    }
    CK(launch_sfactor(a, h->st));
    h->launches += 2;
    return ESP_OK;
}

// Measurements made by their own kernels after measurement `step`: spin
// correlations and the structure factor.
int extra_measure(esp_handle *h, long long step)
{
    int rc = ESP_OK;
    if (h->sc_B && (rc = spincorr_measure(h))) return rc;
    if (h->sf_nq && (rc = sfactor_measure(h, step))) return rc;
    return rc;
}

int measure(esp_handle *h, long long step, int nlev, bool pt_quirk, long long &const_hits)
{
    int rc0 = arrays_current(h);
    if (rc0) return rc0;
    int rc = fold(h);
    if (rc) return rc;
    MeasureArgs m;
    m.e_run = h->d_e_run; m.m_run = h->d_m_run; m.repl_at = h->d_repl_at;
    m.data = h->d_data; m.lsum = h->d_lsum; m.binning = h->d_bin; m.levels = h->d_levels;
    m.R = h->R; m.N = h->N; m.nlev = nlev; m.pt_quirk = pt_quirk ? 1 : 0; m.step = step;
    m.series = h->d_series; m.series_cap = h->series_cap;
    m.ctr = nullptr;
    if (h->capturing) {
        m.step -= h->cap_base[2];
        m.ctr = h->d_ctr + 2;
    }
    m.obs = h->obs;
    m.obs_rep = h->d_obs_rep; m.obs_data = h->d_obs_data; m.obs_lsum = h->d_obs_lsum; m.obs_bin = h->d_obs_bin;
    if (h->obs) {
        // orderparam_get / staggered_get sums of every replica (the energy
        // scratch is free between energy evaluations)
        ObsArgs oa;
        oa.sx = h->d_sx; oa.sy = h->d_sy; oa.sz = h->d_sz; oa.perm = h->d_perm; oa.atom = h->d_obs_atom;
        oa.scratch = h->d_scratch; oa.N = h->N; oa.R = h->R; oa.num_atoms = h->na;
        CK(launch_obs(oa, h->d_obs_rep, h->d_obs_rep + h->R, h->e_blocks, h->st));
        h->launches += 2;
    }
    CK(launch_measure(m, h->st));
    h->launches++;
    {
        int rc = extra_measure(h, step);
        if (rc) return rc;
    }
    // one atom per cell: |sum_cell s| = |m| for every cell, so every cell
    // lands in the top bin of Pm_get's grid; count it without a pass.
    if (h->na == 1) const_hits++;
    if (h->na > 1 || h->obs) {
        PmArgs p;
        p.sx = h->d_sx; p.sy = h->d_sy; p.sz = h->d_sz; p.inv = h->d_inv; p.temp_of = h->d_temp_of;
        p.counts = h->d_pm; p.R = h->R; p.ncell = h->N / h->na; p.num_atoms = h->na; p.nf = h->nf;
        p.use_shared = 0; p.m_min = h->m_min; p.m_max = h->m_max;
        p.count_m = h->na > 1 ? 1 : 0;
        p.obs = h->obs; p.obs_atom = h->d_obs_atom; p.obs_counts = h->d_obs_pm;
        CK(launch_pm(p, h->max_blocks, h->st));
        h->launches++;
    }
    return ESP_OK;
}

int ensure_levels(esp_handle *h, int nlev, const int32_t *levels)
{
    if (nlev > h->nlev_alloc) {
        dfree(h->d_lsum); dfree(h->d_bin); dfree(h->d_levels); dfree(h->d_obs_lsum); dfree(h->d_obs_bin);
        CK(dalloc(&h->d_lsum, (size_t)h->R * nlev * 2));
        CK(dalloc(&h->d_bin, (size_t)h->R * nlev * 2));
        CK(dalloc(&h->d_obs_lsum, (size_t)h->R * nlev * 2));
        CK(dalloc(&h->d_obs_bin, (size_t)h->R * nlev * 2));
        CK(dalloc(&h->d_levels, (size_t)nlev));
        h->nlev_alloc = nlev;
    }
    if (nlev > 0) {
        CK(cudaMemcpyAsync(h->d_levels, levels, sizeof(int32_t) * nlev, cudaMemcpyHostToDevice, h->st));
        CK(cudaMemsetAsync(h->d_lsum, 0, sizeof(double) * h->R * nlev * 2, h->st));
        CK(cudaMemsetAsync(h->d_bin, 0, sizeof(double) * h->R * nlev * 2, h->st));
        CK(cudaMemsetAsync(h->d_obs_lsum, 0, sizeof(double) * h->R * nlev * 2, h->st));
        CK(cudaMemsetAsync(h->d_obs_bin, 0, sizeof(double) * h->R * nlev * 2, h->st));
    }
    return ESP_OK;
}

int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Copies on the handle's stream (which may be non-blocking with respect to
// the legacy default stream), completed before returning.
int h2d(esp_handle *h, void *dst, const void *src, size_t bytes)
{
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
    return ESP_OK;
}

int d2h(esp_handle *h, void *dst, const void *src, size_t bytes)
{
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    return ESP_OK;
}

// Split of Lz planes into cs slabs of an even number of planes, as equal as
// possible: nA slabs of pz planes, cs - nA of pz - 2 (nA == cs: all equal).
bool slab_split(int Lz, int cs, int &pz, int &nA)
{
    if (Lz % 2 != 0 || cs < 1) return false;
    const int pairs = Lz / 2, q = pairs / cs, rem = pairs % cs;
    if (q < 1) return false;
    pz = 2 * (rem ? q + 1 : q);
    nA = rem ? rem : cs;
    return true;
}

// Cluster geometries the GPU can run, cheapest first by a model: cs CTAs of
// nt threads per replica, slabs of an even number of z planes (as equal as
// possible), shared memory within the per-CTA limit; cost = waves of R
// clusters (occupancy calculator) x CTAs one SM holds per wave x the length of
// a sweep in colour passes of the largest slab.
struct ClusterGeom {
    int cs, nt, S;
    double cost;
};

std::vector<ClusterGeom> cluster_candidates(const esp_handle *h)
{
    std::vector<ClusterGeom> out;
    if (!h->d_stencil_blob) return out;
    std::vector<int> per_colour;   // classes of each colour
    for (int k = 0; k < (int)h->prep.class_colour.size(); ++k) {
        const int c = h->prep.class_colour[k];
        if (c >= (int)per_colour.size()) per_colour.resize(c + 1, 0);
        ++per_colour[c];
    }
    const int geoms[3][2] = {{512, 1}, {512, 2}, {256, 1}};   // threads, sites per thread
    for (const auto &tg : geoms)
        for (int cs = 1; cs <= 16; ++cs) {
            const int nt = tg[0], S = tg[1];
            int pz = 0, nA = 0;
            if (!slab_split(h->L[2], cs, pz, nA)) continue;
            // the largest slab sets the shared memory and the pace
            const int n_big = (h->L[0] / 2) * (h->L[1] / 2) * (pz / 2) * 8 * h->na;
            const size_t smem = cluster_smem_bytes(n_big, h->nf, h->obs ? 3 : 1, h->cl_sbytes);
            if (smem > 226 * 1024) continue;
            const int active = cluster_max_active(cs, nt, S, smem, h->R);
            if (active <= 0) continue;
            const double waves = std::ceil((double)h->R / (double)active);
            const double conc = (double)std::min(h->R, active) * cs;
            const double per_sm = std::ceil(conc / (double)std::max(1, h->num_sms));
            // colour passes of a sweep; a pass with two sites per thread
            // takes ~1.85 times one with one site (measured)
            const int64_t per_class = (int64_t)(h->L[0] / 2) * (h->L[1] / 2) * (pz / 2);
            double passes = 0.0;
            for (int n : per_colour) passes += (double)ceil_div(n * per_class, (int64_t)S * nt) * (S == 2 ? 1.85 : 1.0);
            out.push_back({cs, nt, S, waves * per_sm * passes});
        }
    std::stable_sort(out.begin(), out.end(), [](const ClusterGeom &a, const ClusterGeom &b) { return a.cost < b.cost; });
    return out;
}

// Tile geometries (edge T cells, G replicas per CTA), cheapest first by a
// model: HBM bytes per site update 12 ((T+2)^3/T^3 + 1), divided by the
// 32-byte-sector use of G contiguous replicas, and scaled up when one launch
// has fewer than two CTAs per SM.  Shared memory stays within two CTAs per SM.
struct TileGeom {
    int T, G;
    int variant;   // 0 one CTA per tile; pipelined persistent CTAs: 1 one per SM, 2 two per SM
    double cost;
};

std::vector<TileGeom> tile_candidates(const esp_handle *h)
{
    std::vector<TileGeom> out;
    if (!h->d_tile_offs) return out;
    const int Gs[5] = {16, 8, 4, 2, 1};
    for (int T = 2; T <= 32; T += 2) {
        if (h->L[0] % (2 * T) || h->L[1] % (2 * T) || h->L[2] % (2 * T)) continue;
        const int ntiles = (h->L[0] / T) * (h->L[1] / T) * (h->L[2] / T);
        for (int G : Gs) {
            if (h->R % G || 256 % G) continue;
            const double b = (double)(T + 2) / T;
            const double bytes = 12.0 * (b * b * b + 1.0) / std::min(1.0, G / 8.0);
            const double items = (double)(ntiles / 8) * (h->R / G);
            // pipelined persistent variants: the copies overlap the updates,
            // within a CTA (one per SM) or across the CTAs of an SM (two of
            // 256 threads, four of 128 for groups of 4 replicas).  The replica
            // groups of one tile go to neighbouring CTAs at about the same
            // time, so groups of 4 do not waste half of each sector; measured
            // on SC 128^3 x 64 they still ran 15% slower than groups of 8
            // (more, shorter items: more box set-up and barriers per update).
            if (tile_p_supported(T, G, h->na)) {
                const int per_sm = G == 4 ? 4 : 2;
                // 228 KB per SM, 1 KB of it reserved per CTA, 96 B static per CTA
                const size_t fits = (size_t)228 * 1024 / per_sm - 1024 - 128;
                if (tile_p_smem_bytes(T, G, h->na, h->tile_maxst, 1) <= fits) {
                    double cost = (G == 4 ? 0.48 : 0.45) * 12.0 * (b * b * b + 1.0);
                    if (items < 4.0 * per_sm * h->num_sms) cost *= 4.0 * per_sm * h->num_sms / items;
                    out.push_back({T, G, 2, cost});
                }
                if (tile_p_smem_bytes(T, G, h->na, h->tile_maxst, 2) <= 226 * 1024) {
                    double cost = 0.5 * bytes;
                    if (items < 4.0 * h->num_sms) cost *= 4.0 * h->num_sms / items;
                    out.push_back({T, G, 1, cost});
                }
            }
            if (tile_smem_bytes(T, G, h->na, h->tile_maxst) <= 113 * 1024) {
                double cost = bytes;
                if (items < 2.0 * h->num_sms) cost *= 2.0 * h->num_sms / items;
                out.push_back({T, G, 0, cost});
            }
        }
    }
    std::stable_sort(out.begin(), out.end(), [](const TileGeom &a, const TileGeom &b) { return a.cost < b.cost; });
    return out;
}

int tile_geometry(esp_handle *h, int T, int G, int variant)
{
    const size_t smem = variant ? tile_p_smem_bytes(T, G, h->na, h->tile_maxst, 3 - variant)
                                : tile_smem_bytes(T, G, h->na, h->tile_maxst);
    if (variant) CK(tile_p_configure(T, G, 3 - variant, smem));
    else CK(tile_configure(smem));
    CK(cudaStreamSynchronize(h->st));
    int rc = fold(h);
    if (rc) return rc;
    const int nt[3] = {h->L[0] / T, h->L[1] / T, h->L[2] / T};
    const int ntiles = nt[0] * nt[1] * nt[2];
    if (ntiles != h->ntiles) {
        // the tiles' slots, then the fold's chunk slots
        const size_t slots = (size_t)(ntiles + tile_fold_chunks(ntiles)) * h->R;
        dfree(h->d_tile_part); dfree(h->d_tile_rej);
        CK(dalloc(&h->d_tile_part, slots * 4));
        CK(dalloc(&h->d_tile_rej, slots));
        CK(cudaMemsetAsync(h->d_tile_part, 0, sizeof(double) * 4 * slots, h->st));
        CK(cudaMemsetAsync(h->d_tile_rej, 0, sizeof(unsigned long long) * slots, h->st));
    }
    if (variant) {
        // as many persistent CTAs as the GPU holds at once
        TileArgs shape{};
        shape.T = T; shape.G = G; shape.na = h->na; shape.R = h->R;
        shape.ntx = nt[0]; shape.nty = nt[1]; shape.ntz = nt[2];
        shape.has_b = h->prep.has_b; shape.has_d = h->prep.has_d;
        CK(tile_p_grid(shape, smem, h->num_sms, 3 - variant, &h->tile_blocks));
    }
    h->tile_T = T; h->tile_G = G; h->tile_variant = variant;
    for (int d = 0; d < 3; ++d) h->tile_nt[d] = nt[d];
    h->ntiles = ntiles;
    h->tile_smem = smem;
    h->tile_ok = true;
    return ESP_OK;
}

// Stencil offsets of the tiled path, if every entry stays within one cell.
int tile_setup(esp_handle *h)
{
    // per atom: entries with biquadratic or DM couplings first, then
    // exchange-only ones, each part padded to a multiple of 8 with the site
    // itself and zero couplings (the kernels apply the B/D arithmetic to the
    // first part only)
    std::vector<std::vector<StencilEntry>> bd(h->na), jo(h->na);
    int maxst = 8;
    for (int at = 0; at < h->na; ++at) {
        for (const StencilEntry &x : h->prep.stencil[at]) {
            if (std::abs(x.dx) > 1 || std::abs(x.dy) > 1 || std::abs(x.dz) > 1) return ESP_OK;
            const bool rich = x.B != 0.f || x.Dx != 0.f || x.Dy != 0.f || x.Dz != 0.f;
            (rich ? bd[at] : jo[at]).push_back(x);
        }
        h->tile_nbd8[at] = ((int)bd[at].size() + 7) & ~7;
        h->tile_nall8[at] = h->tile_nbd8[at] + (((int)jo[at].size() + 7) & ~7);
        h->tile_nbd2[at] = ((int)bd[at].size() + 1) & ~1;
        h->tile_nall4[at] = h->tile_nbd8[at] + (((int)jo[at].size() + 3) & ~3);
        maxst = std::max(maxst, h->tile_nall8[at]);
    }
    for (int at = h->na; at < kMaxClusterAtoms; ++at)
        h->tile_nbd8[at] = h->tile_nall8[at] = h->tile_nbd2[at] = h->tile_nall4[at] = 0;
    std::vector<int4> offs((size_t)h->na * maxst);
    std::vector<ClusterNbr> cpl((size_t)h->na * maxst);
    for (int at = 0; at < h->na; ++at) {
        for (int e = 0; e < maxst; ++e) {
            offs[(size_t)at * maxst + e] = make_int4(0, 0, 0, at);
            ClusterNbr z{};
            cpl[(size_t)at * maxst + e] = z;
        }
        auto put = [&](int e, const StencilEntry &x) {
            offs[(size_t)at * maxst + e] = make_int4(x.dx, x.dy, x.dz, x.b);
            ClusterNbr &c = cpl[(size_t)at * maxst + e];
            c.J = x.J; c.B = x.B; c.Dx = x.Dx; c.Dy = x.Dy; c.Dz = x.Dz;
        };
        for (size_t e = 0; e < bd[at].size(); ++e) put((int)e, bd[at][e]);
        for (size_t e = 0; e < jo[at].size(); ++e) put(h->tile_nbd8[at] + (int)e, jo[at][e]);
    }
    h->tile_maxst = maxst;
    CK(dalloc(&h->d_tile_offs, offs.size()));
    CK(dalloc(&h->d_tile_cpl, cpl.size()));
    int rc = h2d(h, h->d_tile_offs, offs.data(), sizeof(int4) * offs.size());
    if (rc) return rc;
    if ((rc = h2d(h, h->d_tile_cpl, cpl.data(), sizeof(ClusterNbr) * cpl.size()))) return rc;
    const std::vector<TileGeom> c = tile_candidates(h);
    if (c.empty()) return ESP_OK;
    return tile_geometry(h, c[0].T, c[0].G, c[0].variant);
}

// Set up the cluster path for cs CTAs of nt threads: slab height, shared
// memory, the neighbour table of every CTA rank.
int cluster_geometry(esp_handle *h, int cs, int nt, int S)
{
    // a slab copy of the old geometry goes back to the arrays first
    if (h->cluster_ok) {
        int rc0 = arrays_current(h);
        if (rc0) return rc0;
    }
    const int maxst = h->cl_maxst;
    int pz = 0, nA = 0;
    if (!slab_split(h->L[2], cs, pz, nA)) {
        h->err = "no slab split of the supercell's z planes over this cluster size";
        return ESP_EINVAL;
    }
    const int Lx = h->L[0], Ly = h->L[1], Lz = h->L[2], Hx = Lx / 2, Hy = Ly / 2;
    const int nclass = 8 * h->na;
    const int n_big = Hx * Hy * (pz / 2) * nclass;
    const size_t smem = cluster_smem_bytes(n_big, h->nf, h->obs ? 3 : 1, h->cl_sbytes);
    CK(cluster_configure(smem, cs, nt, S));
    // rank of plane z
    std::vector<int> owner(Lz);
    for (int q = 0; q < cs; ++q)
        for (int z = slab_z0(pz, nA, q); z < slab_z0(pz, nA, q) + slab_planes(pz, nA, q); ++z) owner[z] = q;
    // stencil entry e of local site l on rank q: its local index, with
    // 0x80000000 | (owner rank << 24) when the owner is another rank; stored
    // as [q][e / 4][l][e % 4] (the ranks' blocks one after another) so a
    // thread reads four entries in one 16-byte load
    std::vector<uint32_t> tab((size_t)maxst * h->N);
    for (int q = 0; q < cs; ++q) {
        const int z0 = slab_z0(pz, nA, q), per_class = Hx * Hy * (slab_planes(pz, nA, q) / 2);
        const int n_local = per_class * nclass;
        const size_t base = (size_t)maxst * (size_t)(z0 / 2) * Hx * Hy * nclass;   // in entries
        for (int l = 0; l < n_local; ++l) {
            const int k = l / per_class, rem = l % per_class;
            const int hx = rem % Hx, hy = (rem / Hx) % Hy, hzl = rem / (Hx * Hy);
            const int at = k >> 3, px = (k >> 2) & 1, py = (k >> 1) & 1, pzb = k & 1;
            const int x = 2 * hx + px, y = 2 * hy + py, z = z0 + 2 * hzl + pzb;
            const auto &lst = h->prep.stencil[at];
            for (int e = 0; e < maxst; ++e) {
                uint32_t v = (uint32_t)l;  // padding: the site itself
                if (e < (int)lst.size()) {
                    const StencilEntry &se = lst[e];
                    const int xn = ((x + se.dx) % Lx + Lx) % Lx, yn = ((y + se.dy) % Ly + Ly) % Ly;
                    const int zn = ((z + se.dz) % Lz + Lz) % Lz;
                    const int kn = (se.b << 3) | ((xn & 1) << 2) | ((yn & 1) << 1) | (zn & 1);
                    const int rn = owner[zn];
                    const int pcn = Hx * Hy * (slab_planes(pz, nA, rn) / 2);
                    const int ln = kn * pcn + ((((zn - slab_z0(pz, nA, rn)) >> 1) * Hy + (yn >> 1)) * Hx + (xn >> 1));
                    v = rn == q ? (uint32_t)ln : (0x80000000u | ((uint32_t)rn << 24) | (uint32_t)ln);
                }
                tab[base + (((size_t)(e / 4) * n_local + l) * 4 + e % 4)] = v;
            }
        }
    }
    CK(cudaStreamSynchronize(h->st));
    dfree(h->d_nbidx);
    CK(dalloc(&h->d_nbidx, tab.size()));
    int rc = h2d(h, h->d_nbidx, tab.data(), sizeof(uint32_t) * tab.size());
    if (rc) return rc;
    if (!h->d_slab) CK(dalloc(&h->d_slab, (size_t)3 * h->N * h->R));
    h->csize = cs;
    h->cthreads = nt;
    h->csites = S;
    h->pz = pz;
    h->cl_nA = nA;
    h->cluster_smem = smem;
    h->cluster_ok = true;
    h->slab_ok = false;   // slabs of this geometry are made from the arrays when needed
    return ESP_OK;
}

// Which spin transfers read / write the caller's array directly (bit 0 / 1)
// where the device can.  None by default: measured on a GB300 with a
// coherent CPU link, the device read the caller's array at ~45 GB/s against
// ~38 GB/s staged, and wrote freshly allocated (not yet touched) pages at
// 2.7 GB/s, faulting each in, against ~26 GB/s staged.
constexpr int kHostTransferDefault = 0;
int host_transfer_mode(const esp_handle *h)
{
    if (!h->host_direct_ok) return 0;
    return h->host_transfer >= 0 ? h->host_transfer : kHostTransferDefault;
}

// Staging for spin_matrix blocks of whole temperature slots, at most 256 MiB
// (one slot at least), on the device and in pinned host memory; allocated
// with the tables so that the spin transfers themselves allocate nothing.
int ensure_stage(esp_handle *h)
{
    if (h->d_stage && h->h_stage && h->stage_slots > 0 && h->stage_ev[0] && h->stage_ev[1]) return ESP_OK;
    // set up both halves or neither: a handle left with one of them would
    // loop forever over zero-slot blocks in esp_set_spins / esp_get_spins
    dfree(h->d_stage);
    if (h->h_stage) cudaFreeHost(h->h_stage);
    h->h_stage = nullptr;
    h->stage_slots = 0;
    const size_t per_slot = sizeof(double) * 3 * (size_t)h->N;
    int slots = (int)std::max<size_t>(1, ((size_t)256 << 20) / per_slot);
    slots = std::min(slots, h->R);
    CK(dalloc(&h->d_stage, (size_t)3 * h->N * slots));
    cudaError_t e = cudaMallocHost((void **)&h->h_stage, sizeof(double) * 3 * (size_t)h->N * slots);
    if (e != cudaSuccess) {
        dfree(h->d_stage);
        h->h_stage = nullptr;
        h->err = std::string("cudaMallocHost of the spin staging: ") + cudaGetErrorString(e);
        return ESP_ENOMEM;
    }
    for (cudaEvent_t &ev : h->stage_ev) {
        if (!ev && (e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess) {
            dfree(h->d_stage);
            cudaFreeHost(h->h_stage);
            h->h_stage = nullptr;
            h->err = std::string("cudaEventCreate: ") + cudaGetErrorString(e);
            return ESP_ECUDA;
        }
    }
    h->stage_slots = slots;
    return ESP_OK;
}

// The staging as two halves of `half` slots each (one half, the whole
// staging, when it holds a single slot): the host copy of one block runs while
// the other half's block crosses the link and is converted on the device.
int stage_half(const esp_handle *h) { return h->stage_slots >= 2 ? h->stage_slots / 2 : h->stage_slots; }

// Host copy between the caller's arrays and the pinned staging, split over
// up to 16 threads (the host's cores) for large blocks: one core copies (and
// faults in fresh pages) far below the memory bandwidth.
void par_memcpy(void *dst, const void *src, size_t bytes)
{
    const size_t chunk = (size_t)4 << 20;
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int nth = (int)std::min<size_t>(std::min(16u, hw), bytes / chunk);
    if (nth <= 1) {
        std::memcpy(dst, src, bytes);
        return;
    }
    const size_t per = ((bytes + nth - 1) / nth + 63) & ~(size_t)63;
    std::vector<std::thread> th;
    th.reserve(nth - 1);
    for (int i = 1; i < nth; ++i) {
        const size_t off = per * i;
        if (off >= bytes) break;
        const size_t n = std::min(per, bytes - off);
        th.emplace_back([=] { std::memcpy(static_cast<char *>(dst) + off, static_cast<const char *>(src) + off, n); });
    }
    std::memcpy(dst, src, std::min(per, bytes));
    for (std::thread &t : th) t.join();
}

}  // namespace

namespace esp {
void set_global_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_global_err, sizeof(g_global_err), fmt, ap);
    va_end(ap);
}
}  // namespace esp

extern "C" {

int esp_create(const esp_dims *dims, esp_handle **out)
{
    if (!dims || !out) { set_global_error("null argument"); return ESP_EINVAL; }
    *out = nullptr;
    if (dims->num_sites <= 0 || dims->num_atoms <= 0 || dims->num_replicas <= 0 ||
        dims->supercell[0] <= 0 || dims->supercell[1] <= 0 || dims->supercell[2] <= 0) {
        set_global_error("dimensions must be positive");
        return ESP_EINVAL;
    }
    if ((long long)dims->supercell[0] * dims->supercell[1] * dims->supercell[2] * dims->num_atoms != dims->num_sites) {
        set_global_error("num_sites != prod(supercell) * num_atoms");
        return ESP_EINVAL;
    }
    esp_handle *h = new (std::nothrow) esp_handle();
    if (!h) { set_global_error("host allocation failed"); return ESP_ENOMEM; }
    h->N = dims->num_sites; h->R = dims->num_replicas; h->na = dims->num_atoms;
    for (int c = 0; c < 3; ++c) h->L[c] = dims->supercell[c];
    h->open = dims->open_boundary != 0;
    cudaError_t e = cudaGetDevice(&h->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device);
    if (e == cudaSuccess) {
        int pageable = 0, host_tables = 0;
        if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, h->device) != cudaSuccess) pageable = 0;
        if (cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, h->device) !=
            cudaSuccess)
            host_tables = 0;
        h->host_direct_ok = pageable == 1 && host_tables == 1;
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->own, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = lp_configure(h->device);
    if (e == cudaSuccess) e = lp_tc_configure();
    if (e == cudaSuccess) e = lp_tc_sweep_configure();
    if (e == cudaSuccess) e = gemm_tc_configure();
    if (e != cudaSuccess) {
        set_global_error("CUDA unavailable: %s", cudaGetErrorString(e));
        delete h;
        return ESP_ECUDA;
    }
    h->st = h->own;
    h->max_blocks = h->num_sms * 8;
    const size_t NR = (size_t)h->N * h->R;
    e = cudaSuccess;
    if (e == cudaSuccess) e = dalloc(&h->d_sx, NR);
    if (e == cudaSuccess) e = dalloc(&h->d_sy, NR);
    if (e == cudaSuccess) e = dalloc(&h->d_sz, NR);
    if (e == cudaSuccess) e = dalloc(&h->d_temp_of, h->R);
    if (e == cudaSuccess) e = dalloc(&h->d_repl_at, h->R);
    if (e == cudaSuccess) e = dalloc(&h->d_beta, h->R);
    if (e == cudaSuccess) e = dalloc(&h->d_inv_t, h->R);
    if (e == cudaSuccess) e = dalloc(&h->d_e_run, h->R);
    if (e == cudaSuccess) e = dalloc(&h->d_m_run, 3 * (size_t)h->R);
    if (e == cudaSuccess) e = dalloc(&h->d_rej, 2 * (size_t)h->R);
    if (e == cudaSuccess) e = dalloc(&h->d_tmp_e, h->R);
    if (e == cudaSuccess) e = dalloc(&h->d_tmp_m, 3 * (size_t)h->R);
    if (e == cudaSuccess) e = dalloc(&h->d_data, 6 * (size_t)h->R);
    if (e == cudaSuccess) e = dalloc(&h->d_swaps, 2 * (size_t)h->R);
    if (e != cudaSuccess) {
        set_global_error("device allocation failed: %s", cudaGetErrorString(e));
        free_all(h);
        cudaStreamDestroy(h->own);
        delete h;
        return ESP_ENOMEM;
    }
    cudaMemset(h->d_rej, 0, sizeof(unsigned long long) * 2 * h->R);
    cudaMemset(h->d_e_run, 0, sizeof(double) * h->R);
    cudaMemset(h->d_m_run, 0, sizeof(double) * 3 * h->R);
    *out = h;
    return identity_labels(h);
}

int esp_destroy(esp_handle *h)
{
    if (!h) return ESP_EINVAL;
    if (h->st) cudaStreamSynchronize(h->st);
    free_all(h);
    if (h->own) cudaStreamDestroy(h->own);
    delete h;
    return ESP_OK;
}

int esp_last_error(const esp_handle *h, char *buf, size_t len)
{
    if (!buf || len == 0) return ESP_EINVAL;
    std::snprintf(buf, len, "%s", h ? h->err.c_str() : g_global_err);
    return ESP_OK;
}

int esp_set_stream(esp_handle *h, void *stream)
{
    if (!h) return ESP_EINVAL;
    CK(cudaStreamSynchronize(h->st));
    h->st = (cudaStream_t)stream;  // NULL is the legacy default stream
    return ESP_OK;
}

int esp_upload_tables(esp_handle *h, const esp_tables *t)
{
    if (!h || !t) return ESP_EINVAL;
    if (h->cluster_ok) {   // the state back in the arrays before the tables change
        int rc0 = arrays_current(h);
        if (rc0) return rc0;
    }
    h->slab_ok = false;
    PrepInput in;
    in.N = h->N; in.num_atoms = h->na; in.L[0] = h->L[0]; in.L[1] = h->L[1]; in.L[2] = h->L[2];
    in.open_boundary = h->open;
    in.mag = t->mag;
    in.j_maxnb = t->j_maxnb; in.j_nn = t->j_nn; in.j_nbors = t->j_nbors; in.j_val = t->j_val;
    in.b_maxnb = t->b_maxnb; in.b_nn = t->b_nn; in.b_nbors = t->b_nbors; in.b_val = t->b_val;
    in.d_maxnb = t->d_maxnb; in.d_nn = t->d_nn; in.d_nbors = t->d_nbors; in.d_val = t->d_val;
    if (in.b_nn && (!in.b_nbors || !in.b_val)) { h->err = "incomplete bij tables"; return ESP_EINVAL; }
    if (in.d_nn && (!in.d_nbors || !in.d_val)) { h->err = "incomplete dij tables"; return ESP_EINVAL; }
    PrepOutput prep;
    std::string err;
    int rc = prepare_tables(in, prep, err);
    if (rc) { h->err = err; return rc == 2 ? ESP_ECOLOR : ESP_EINVAL; }
    CK(cudaStreamSynchronize(h->st));
    free_tables(h);
    free_obs(h);
    free_sc(h);
    free_sf(h);
    h->have_tables = false;
    h->mag_host.assign(t->mag, t->mag + h->N);
    const size_t M = (size_t)prep.maxnb * h->N;
    CK(dalloc(&h->d_nnb, h->N));
    CK(dalloc(&h->d_nbr, M));
    CK(dalloc(&h->d_perm, h->N));
    CK(dalloc(&h->d_inv, h->N));
    CK(dalloc(&h->d_J, M));
    CK(dalloc(&h->d_mag, h->N));
    if ((rc = h2d(h, h->d_nnb, prep.nnb.data(), sizeof(int32_t) * h->N))) return rc;
    if ((rc = h2d(h, h->d_nbr, prep.nbr.data(), sizeof(int32_t) * M))) return rc;
    if ((rc = h2d(h, h->d_perm, prep.perm.data(), sizeof(int32_t) * h->N))) return rc;
    if ((rc = h2d(h, h->d_inv, prep.inv.data(), sizeof(int32_t) * h->N))) return rc;
    if ((rc = h2d(h, h->d_J, prep.J.data(), sizeof(float) * M))) return rc;
    if ((rc = h2d(h, h->d_mag, prep.mag.data(), sizeof(float) * h->N))) return rc;
    if (prep.has_b) {
        CK(dalloc(&h->d_B, M));
        if ((rc = h2d(h, h->d_B, prep.B.data(), sizeof(float) * M))) return rc;
    }
    if (prep.has_d) {
        CK(dalloc(&h->d_Dx, M)); CK(dalloc(&h->d_Dy, M)); CK(dalloc(&h->d_Dz, M));
        if ((rc = h2d(h, h->d_Dx, prep.Dx.data(), sizeof(float) * M))) return rc;
        if ((rc = h2d(h, h->d_Dy, prep.Dy.data(), sizeof(float) * M))) return rc;
        if ((rc = h2d(h, h->d_Dz, prep.Dz.data(), sizeof(float) * M))) return rc;
    }
    h->hsi = t->si_axis != nullptr && t->si_delta != nullptr;
    h->hfld = t->field_axis != nullptr && t->field_val != nullptr;
    std::vector<float4> si(h->na), fl(h->na);
    for (int a = 0; a < h->na; ++a) {
        if (h->hsi)
            si[a] = make_float4((float)t->si_axis[3 * a], (float)t->si_axis[3 * a + 1], (float)t->si_axis[3 * a + 2],
                                (float)t->si_delta[a]);
        if (h->hfld)
            fl[a] = make_float4((float)(t->field_val[a] * t->field_axis[3 * a]),
                                (float)(t->field_val[a] * t->field_axis[3 * a + 1]),
                                (float)(t->field_val[a] * t->field_axis[3 * a + 2]), 0.f);
    }
    CK(dalloc(&h->d_si, h->na));
    CK(dalloc(&h->d_fld, h->na));
    if ((rc = h2d(h, h->d_si, si.data(), sizeof(float4) * h->na))) return rc;
    if ((rc = h2d(h, h->d_fld, fl.data(), sizeof(float4) * h->na))) return rc;
    // reference axis of the learned proposal's local frame: the single-ion axis
    CK(dalloc(&h->d_lp_axis, h->na));
    if ((rc = h2d(h, h->d_lp_axis, si.data(), sizeof(float4) * h->na))) return rc;
    {
        int maxc = 0;
        for (int c = 0; c < prep.num_colours; ++c) maxc = std::max(maxc, prep.off[c + 1] - prep.off[c]);
        h->sweep_grid = sweep_blocks((long long)maxc * h->R, h->R, h->max_blocks);
        h->slots = std::min(h->R, 256);
        // the learned sweep's 512-thread blocks count as two 256-thread blocks
        h->lp_grid = lp_sweep_blocks((long long)maxc * h->R, h->R, h->num_sms);
        h->part_blocks = std::max(h->sweep_grid, 2 * h->lp_grid);
        h->tc_grid = lp_tc_sweep_blocks((long long)maxc * h->R, h->R, h->num_sms);
        h->tc_slots = std::min(h->R, 128);
        const size_t tslot = (size_t)h->tc_grid * h->tc_slots;
        CK(dalloc(&h->d_tc_part, 4 * tslot));
        CK(dalloc(&h->d_tc_part_rej, tslot));
        CK(cudaMemsetAsync(h->d_tc_part, 0, sizeof(double) * 4 * tslot, h->st));
        CK(cudaMemsetAsync(h->d_tc_part_rej, 0, sizeof(unsigned long long) * tslot, h->st));
        h->tc_pending = 0;
        const size_t nslot = (size_t)h->part_blocks * h->slots;
        CK(dalloc(&h->d_part, 4 * nslot));
        CK(dalloc(&h->d_part_rej, nslot));
        CK(cudaMemsetAsync(h->d_part, 0, sizeof(double) * 4 * nslot, h->st));
        CK(cudaMemsetAsync(h->d_part_rej, 0, sizeof(unsigned long long) * nslot, h->st));
        h->pending_sweeps = 0;
    }
    // P(M) grid (mcarlo.F90:432-442)
    double mmax = 0.0;
    for (int a = 0; a < h->na; ++a) mmax += std::fabs(t->mag[a]);
    h->m_max = mmax; h->m_min = -mmax;
    h->nf = (int)std::llround((h->m_max - h->m_min) / 0.01) + 1;
    if (h->nf == 1) h->nf = 2;
    // cluster-resident path: translation-invariant lattice whose replica fits
    // in the distributed shared memory of one cluster
    h->cluster_ok = false;
    if (prep.invariant && h->na <= kMaxClusterAtoms && prep.num_colours <= kMaxClasses &&
        (int)prep.class_colour.size() == 8 * h->na && h->L[0] % 2 == 0 && h->L[1] % 2 == 0 && h->L[2] % 2 == 0) {
        const int nclass = 8 * h->na;
        int maxst = 0;
        for (int at = 0; at < h->na; ++at) maxst = std::max(maxst, (int)prep.stencil[at].size());
        maxst = (maxst + 7) & ~7;  // the kernel reads neighbours in groups of 8
        const size_t sbytes = (cluster_stencil_bytes(nclass, maxst) + 15) & ~(size_t)15;
        std::vector<unsigned char> blob(sbytes, 0);
        ClusterStencil &hs = *reinterpret_cast<ClusterStencil *>(blob.data());
        ClusterNbr *nbs = reinterpret_cast<ClusterNbr *>(blob.data() + sizeof(ClusterStencil));
        bool fits = true;
        hs.nclass = nclass; hs.maxst = maxst; hs.ncolour = prep.num_colours;
        for (int k = 0; k < nclass; ++k) {
            const int at = k >> 3;
            const auto &lst = prep.stencil[at];
            hs.count[k] = (int)lst.size();
            for (size_t e = 0; e < lst.size(); ++e) {
                const StencilEntry &x = lst[e];
                ClusterNbr &nb = nbs[(size_t)k * maxst + e];
                nb.J = x.J; nb.B = x.B; nb.Dx = x.Dx; nb.Dy = x.Dy; nb.Dz = x.Dz;
            }
        }
        for (int at = 0; at < h->na; ++at) {
            if (h->hsi)
                hs.si[at] = make_float4((float)t->si_axis[3 * at], (float)t->si_axis[3 * at + 1],
                                        (float)t->si_axis[3 * at + 2], (float)t->si_delta[at]);
            if (h->hfld)
                hs.fld[at] = make_float4((float)(t->field_val[at] * t->field_axis[3 * at]),
                                         (float)(t->field_val[at] * t->field_axis[3 * at + 1]),
                                         (float)(t->field_val[at] * t->field_axis[3 * at + 2]), 0.f);
            hs.mag[at] = (float)t->mag[at];
        }
        // every site of an atom must carry that atom's moment
        for (int i = 0; i < h->N && fits; ++i)
            if ((float)t->mag[i] != hs.mag[i % h->na]) fits = false;
        {
            int n = 0;
            for (int c = 0; c < prep.num_colours; ++c) {
                hs.colour_start[c] = n;
                for (int k = 0; k < nclass; ++k)
                    if (prep.class_colour[k] == c) hs.class_order[n++] = k;
            }
            hs.colour_start[prep.num_colours] = n;
        }
        if (fits) {
            h->cl_maxst = maxst;
            h->cl_sbytes = sbytes;
            h->stencil_words = (int)(sbytes / 4);
            CK(dalloc(&h->d_stencil_blob, sbytes));
            if ((rc = h2d(h, h->d_stencil_blob, blob.data(), sbytes))) return rc;
        }
    }
    h->e_blocks = energy_blocks(h->N, h->R, h->max_blocks);
    CK(dalloc(&h->d_scratch, (size_t)h->e_blocks * h->R * 4));
    dfree(h->d_pm);
    CK(dalloc(&h->d_pm, (size_t)h->R * h->nf));
    h->prep = std::move(prep);
    h->ntiles = 0;
    if (h->d_stencil_blob) {
        const std::vector<ClusterGeom> c = cluster_candidates(h);
        if (!c.empty() && (rc = cluster_geometry(h, c[0].cs, c[0].nt, c[0].S))) return rc;
        if ((rc = tile_setup(h))) return rc;
    }
    if ((rc = ensure_stage(h))) return rc;
    h->have_tables = true;
    return ESP_OK;
}

int esp_set_temperatures(esp_handle *h, const double *tems)
{
    if (!h || !tems) return ESP_EINVAL;
    std::vector<float> beta(h->R);
    std::vector<double> inv(h->R);
    for (int t = 0; t < h->R; ++t) {
        if (!(tems[t] > 0.0)) { h->err = "temperatures must be positive"; return ESP_EINVAL; }
        beta[t] = (float)(1.0 / tems[t]);
        inv[t] = 1.0 / tems[t];
    }
    h->tems.assign(tems, tems + h->R);
    CK(cudaMemcpyAsync(h->d_beta, beta.data(), sizeof(float) * h->R, cudaMemcpyHostToDevice, h->st));
    CK(cudaMemcpyAsync(h->d_inv_t, inv.data(), sizeof(double) * h->R, cudaMemcpyHostToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
    h->have_temps = true;
    return identity_labels(h);
}

int esp_set_spins(esp_handle *h, const double *spins)
{
    int rc = require(h, true, false);
    if (rc) return rc;
    if (!spins) { h->err = "null spins"; return ESP_EINVAL; }
    if ((rc = ensure_stage(h))) return rc;
    arrays_written(h);   // every slot is overwritten below
    if (host_transfer_mode(h) & 1) {
        // one kernel reads the caller's FP64 array over the CPU-GPU link
        CK(launch_spins_in(spins, h->d_inv, h->d_repl_at, h->d_sx, h->d_sy, h->d_sz, h->N, h->R, 0, h->R, h->st));
        h->launches++;
        if ((rc = reset_running(h))) return rc;
        CK(cudaStreamSynchronize(h->st));
        return ESP_OK;
    }
    // blocks of slots: copy the FP64 block through the pinned staging (a
    // parallel host copy, then one DMA), then scatter it into the permuted
    // FP32 state on the device; the blocks alternate between the staging's
    // halves, so the host copy of one overlaps the DMA and conversion of the
    // previous.  The driver's pageable path is as fast only for warm, small
    // arrays and falls to ~1 GB/s where it must fault pages in.
    const int half = stage_half(h);
    const size_t half_el = (size_t)3 * h->N * half;
    CK(cudaStreamSynchronize(h->st));   // the halves' events belong to this call from here on
    for (int t0 = 0, k = 0; t0 < h->R; t0 += half, ++k) {
        const int nt = std::min(half, h->R - t0), b = h->stage_slots >= 2 ? (k & 1) : 0;
        const size_t bytes = sizeof(double) * 3 * (size_t)h->N * nt;
        if (k >= (h->stage_slots >= 2 ? 2 : 1))
            CK(cudaEventSynchronize(h->stage_ev[b]));   // this half's previous block has left the pinned memory
        par_memcpy(h->h_stage + b * half_el, spins + (size_t)3 * h->N * t0, bytes);
        CK(cudaMemcpyAsync(h->d_stage + b * half_el, h->h_stage + b * half_el, bytes, cudaMemcpyHostToDevice,
                           h->st));
        CK(cudaEventRecord(h->stage_ev[b], h->st));
        CK(launch_spins_in(h->d_stage + b * half_el, h->d_inv, h->d_repl_at, h->d_sx, h->d_sy, h->d_sz, h->N, h->R,
                           t0, nt, h->st));
        h->launches++;
    }
    if ((rc = reset_running(h))) return rc;
    CK(cudaStreamSynchronize(h->st));
    return ESP_OK;
}

int esp_init_spins(esp_handle *h, int32_t kind, uint64_t seed)
{
    int rc = require(h, true, false);
    if (rc) return rc;
    if (kind != 0 && kind != 1) { h->err = "kind must be 0 (ferro) or 1 (rand)"; return ESP_EINVAL; }
    arrays_written(h);
    CK(launch_init_spins(h->d_perm, h->d_mag, h->d_sx, h->d_sy, h->d_sz, h->N, h->R, kind, seed, h->st));
    h->launches++;
    if ((rc = reset_running(h))) return rc;
    CK(cudaStreamSynchronize(h->st));
    return ESP_OK;
}

int esp_get_spins(esp_handle *h, double *spins)
{
    int rc = require(h, true, false);
    if (rc) return rc;
    if (!spins) { h->err = "null spins"; return ESP_EINVAL; }
    if ((rc = ensure_stage(h))) return rc;
    if ((rc = arrays_current(h))) return rc;
    if (host_transfer_mode(h) & 2) {
        // one kernel writes the caller's FP64 array over the CPU-GPU link
        CK(launch_spins_out(spins, h->d_inv, h->d_repl_at, h->d_sx, h->d_sy, h->d_sz, h->N, h->R, 0, h->R, h->st));
        h->launches++;
        CK(cudaStreamSynchronize(h->st));
        return ESP_OK;
    }
    // blocks alternate between the staging's halves: block k is gathered and
    // crosses the link while the host copies block k - 1 out of the other half
    const int half = stage_half(h);
    const size_t half_el = (size_t)3 * h->N * half;
    int prev_t0 = -1, prev_b = 0;
    size_t prev_bytes = 0;
    auto drain = [&]() -> int {
        CK(cudaEventSynchronize(h->stage_ev[prev_b]));
        par_memcpy(spins + (size_t)3 * h->N * prev_t0, h->h_stage + prev_b * half_el, prev_bytes);
        prev_t0 = -1;
        return ESP_OK;
    };
    for (int t0 = 0, k = 0; t0 < h->R; t0 += half, ++k) {
        const int nt = std::min(half, h->R - t0), b = h->stage_slots >= 2 ? (k & 1) : 0;
        const size_t bytes = sizeof(double) * 3 * (size_t)h->N * nt;
        if (prev_t0 >= 0 && b == prev_b && (rc = drain())) return rc;   // one half only: empty it first
        CK(launch_spins_out(h->d_stage + b * half_el, h->d_inv, h->d_repl_at, h->d_sx, h->d_sy, h->d_sz, h->N, h->R,
                            t0, nt, h->st));
        h->launches++;
        CK(cudaMemcpyAsync(h->h_stage + b * half_el, h->d_stage + b * half_el, bytes, cudaMemcpyDeviceToHost, h->st));
        CK(cudaEventRecord(h->stage_ev[b], h->st));
        if (prev_t0 >= 0 && (rc = drain())) return rc;
        prev_t0 = t0; prev_b = b; prev_bytes = bytes;
    }
    if (prev_t0 >= 0 && (rc = drain())) return rc;
    return ESP_OK;
}

int esp_sweep(esp_handle *h, int64_t n, int64_t first_sweep, const esp_sweep_opts *o)
{
    int rc = require(h, true, true);
    if (rc) return rc;
    if (!o || n < 0) { h->err = "bad sweep arguments"; return ESP_EINVAL; }
    if ((rc = do_sweeps(h, n, first_sweep, o))) return rc;
    CK(cudaGetLastError());
    return ESP_OK;
}

int esp_sweep_colour(esp_handle *h, int32_t colour, int64_t sweep, const esp_sweep_opts *o)
{
    int rc = require(h, true, true);
    if (rc) return rc;
    if (!o || colour < 0 || colour >= h->prep.num_colours) { h->err = "bad colour"; return ESP_EINVAL; }
    return do_sweep_colour(h, colour, sweep, o);
}

}  // extern "C"

namespace {

// pt_swap of every lattice (group of temperatures); `unit` is the 1-based
// unit index whose parity gives `start` (used when capturing a graph).
int pt_swap_launch(esp_handle *h, int32_t start, int64_t swap_index, uint64_t seed, int64_t unit)
{
    int rc = fold(h);
    if (rc) return rc;
    PtSwapArgs a;
    a.repl_at = h->d_repl_at; a.temp_of = h->d_temp_of; a.e_run = h->d_e_run; a.inv_t = h->d_inv_t;
    a.num_swaps = h->d_swaps; a.R = h->R; a.start0 = start - 1;
    a.group = h->pt_group > 0 ? h->pt_group : h->R;
    a.key0 = (uint32_t)seed; a.key1 = (uint32_t)(seed >> 32);
    a.ctr = nullptr; a.unit_off = 0;
    if (h->capturing) {
        swap_index -= h->cap_base[1];
        a.unit_off = (int32_t)(unit - h->cap_base[3]);
        a.ctr = h->d_ctr;
    }
    a.idx_lo = (uint32_t)swap_index; a.idx_hi = (uint32_t)((uint64_t)swap_index >> 32);
    CK(launch_pt_swap(a, h->st));
    h->launches++;
    return ESP_OK;
}

}  // namespace

extern "C" {

int esp_pt_swap(esp_handle *h, int32_t start, int64_t swap_index, uint64_t seed)
{
    int rc = require(h, true, true);
    if (rc) return rc;
    if (start != 1 && start != 2) { h->err = "start must be 1 or 2"; return ESP_EINVAL; }
    return pt_swap_launch(h, start, swap_index, seed, 0);
}

int esp_set_pt_groups(esp_handle *h, int32_t group_size)
{
    if (!h) return ESP_EINVAL;
    if (group_size < 1 || h->R % group_size != 0) {
        h->err = "the PT group size must divide the number of replicas";
        return ESP_EINVAL;
    }
    int rc = fold(h);
    if (rc) return rc;
    h->pt_group = group_size;
    return ESP_OK;
}

int esp_energy(esp_handle *h, double *energy_out)
{
    int rc = require(h, true, false);
    if (rc) return rc;
    if ((rc = reset_running(h))) return rc;
    if (energy_out) return by_slot(h, h->d_tmp_e, 1, energy_out);
    CK(cudaStreamSynchronize(h->st));
    return ESP_OK;
}

int esp_running_energy(esp_handle *h, double *out)
{
    int rc = require(h, true, false);
    if (rc) return rc;
    if ((rc = fold(h))) return rc;
    return by_slot(h, h->d_e_run, 1, out);
}

int esp_running_magnetization(esp_handle *h, double *out)
{
    int rc = require(h, true, false);
    if (rc) return rc;
    if ((rc = fold(h))) return rc;
    return by_slot(h, h->d_m_run, 3, out);
}

int esp_local_terms(esp_handle *h, double *g_out, double *q_out)
{
    int rc = require(h, true, false);
    if (rc) return rc;
    if ((rc = arrays_current(h))) return rc;
    const size_t NR = (size_t)h->N * h->R;
    float *dg = nullptr, *dq = nullptr;
    CK(dalloc(&dg, NR * 3));
    cudaError_t e = dalloc(&dq, NR * 6);
    if (e != cudaSuccess) { cudaFree(dg); h->err = cudaGetErrorString(e); return ESP_ENOMEM; }
    e = launch_local_terms(energy_args(h), dg, dq, h->st);
    h->launches++;
    std::vector<float> g(NR * 3), q(NR * 6);
    if (e == cudaSuccess) e = cudaMemcpyAsync(g.data(), dg, sizeof(float) * NR * 3, cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(q.data(), dq, sizeof(float) * NR * 6, cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    cudaFree(dg); cudaFree(dq);
    if (e != cudaSuccess) { h->err = cudaGetErrorString(e); return ESP_ECUDA; }
    std::vector<int32_t> ra;
    if ((rc = get_repl_at(h, ra))) return rc;
    for (int t = 0; t < h->R; ++t)
        for (int i = 0; i < h->N; ++i) {
            const size_t it = (size_t)h->prep.inv[i] * h->R + ra[t];
            const size_t o = (size_t)t * h->N + i;
            if (g_out) for (int c = 0; c < 3; ++c) g_out[3 * o + c] = g[3 * it + c];
            if (q_out) for (int c = 0; c < 6; ++c) q_out[6 * o + c] = q[6 * it + c];
        }
    return ESP_OK;
}

int esp_get_colouring(esp_handle *h, int32_t *colour_out, int32_t *num_colours)
{
    int rc = require(h, true, false);
    if (rc) return rc;
    if (colour_out) for (int i = 0; i < h->N; ++i) colour_out[i] = h->prep.colour[i];
    if (num_colours) *num_colours = h->prep.num_colours;
    return ESP_OK;
}

int esp_get_rejected(esp_handle *h, int64_t *out)
{
    if (!h || !out) return ESP_EINVAL;
    if (h->have_tables) {
        int rc = fold(h);
        if (rc) return rc;
    }
    CK(cudaMemcpyAsync(out, h->d_rej, sizeof(int64_t) * 2 * h->R, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    return ESP_OK;
}

int esp_get_replica_of_slot(esp_handle *h, int32_t *out)
{
    if (!h || !out) return ESP_EINVAL;
    std::vector<int32_t> ra;
    int rc = get_repl_at(h, ra);
    if (rc) return rc;
    std::copy(ra.begin(), ra.end(), out);
    return ESP_OK;
}

int esp_set_series(esp_handle *h, int64_t capacity)
{
    if (!h || capacity < 0) return ESP_EINVAL;
    CK(cudaStreamSynchronize(h->st));
    dfree(h->d_series);
    h->series_cap = 0;
    if (capacity > 0) {
        CK(dalloc(&h->d_series, (size_t)capacity * h->R * 2));
        h->series_cap = capacity;
    }
    return ESP_OK;
}

int esp_get_series(esp_handle *h, double *out, int64_t *count)
{
    if (!h || !count) return ESP_EINVAL;
    const long long done = h->run.meas_done;
    const long long n = std::min<long long>(done, h->series_cap);
    *count = n;
    if (!out || n == 0) return ESP_OK;
    std::vector<double> all((size_t)h->series_cap * h->R * 2);
    int rc = d2h(h, all.data(), h->d_series, sizeof(double) * all.size());
    if (rc) return rc;
    const long long first = done - n;  // 0-based index of the oldest kept measurement
    for (long long k = 0; k < n; ++k) {
        const long long row = (first + k) % h->series_cap;
        std::memcpy(out + (size_t)k * h->R * 2, all.data() + (size_t)row * h->R * 2, sizeof(double) * h->R * 2);
    }
    return ESP_OK;
}

int esp_set_sweep_kernel(esp_handle *h, int32_t kind)
{
    if (!h || kind < 0 || kind > 4 || kind == 3) return ESP_EINVAL;
    if (kind == 2 && !h->cluster_ok) {
        h->err = "the cluster-resident sweep needs a periodic, translation-invariant lattice that fits a cluster";
        return ESP_EINVAL;
    }
    if (kind == 4 && !h->tile_ok) {
        h->err = "the tiled sweep needs a periodic, translation-invariant lattice with nearest-cell couplings "
                 "and even tile counts";
        return ESP_EINVAL;
    }
    int rc = fold(h);
    if (rc) return rc;
    h->kernel_choice = kind;
    return ESP_OK;
}

int esp_set_tile_geometry(esp_handle *h, int32_t tile, int32_t replicas, int32_t pipelined)
{
    if (!h) return ESP_EINVAL;
    for (const TileGeom &g : tile_candidates(h))
        if (g.T == tile && g.G == replicas && g.variant == pipelined)
            return tile_geometry(h, tile, replicas, g.variant);
    h->err = "tile geometry not possible for this lattice";
    return ESP_EINVAL;
}

int esp_set_host_transfer(esp_handle *h, int32_t mode)
{
    if (!h || mode < -1 || mode > 3) return ESP_EINVAL;
    if (mode > 0 && !h->host_direct_ok) {
        h->err = "the device does not access pageable host memory through the host's page tables";
        return ESP_EINVAL;
    }
    h->host_transfer = mode;
    return ESP_OK;
}

int esp_get_host_transfer(const esp_handle *h, int32_t *mode, int32_t *direct_supported)
{
    if (!h || !mode) return ESP_EINVAL;
    *mode = host_transfer_mode(h);
    if (direct_supported) *direct_supported = h->host_direct_ok ? 1 : 0;
    return ESP_OK;
}

int esp_get_tile_geometry(const esp_handle *h, int32_t *tile, int32_t *replicas, int32_t *pipelined)
{
    if (!h || !tile || !replicas) return ESP_EINVAL;
    *tile = h->tile_ok ? h->tile_T : 0;
    *replicas = h->tile_ok ? h->tile_G : 0;
    if (pipelined) *pipelined = h->tile_ok ? h->tile_variant : 0;
    return ESP_OK;
}

int esp_set_cluster_geometry(esp_handle *h, int32_t cluster_size, int32_t threads, int32_t sites_per_thread)
{
    if (!h) return ESP_EINVAL;
    if (!h->have_tables || !h->d_stencil_blob) {
        h->err = "the cluster-resident sweep needs a periodic, translation-invariant lattice that fits a cluster";
        return ESP_EINVAL;
    }
    for (const ClusterGeom &g : cluster_candidates(h))
        if (g.cs == cluster_size && g.nt == threads && g.S == sites_per_thread) {
            int rc = fold(h);
            if (rc) return rc;
            return cluster_geometry(h, cluster_size, threads, sites_per_thread);
        }
    h->err = "cluster geometry not possible for this lattice on this GPU";
    return ESP_EINVAL;
}

int esp_get_cluster_geometry(const esp_handle *h, int32_t *cluster_size, int32_t *threads, int32_t *sites_per_thread)
{
    if (!h || !cluster_size || !threads) return ESP_EINVAL;
    *cluster_size = h->cluster_ok ? h->csize : 0;
    *threads = h->cluster_ok ? h->cthreads : 0;
    if (sites_per_thread) *sites_per_thread = h->cluster_ok ? h->csites : 0;
    return ESP_OK;
}

int esp_get_sweep_kernel(const esp_handle *h, int32_t *kind, int32_t *cluster_size)
{
    if (!h || !kind) return ESP_EINVAL;
    *kind = h->proposal == 1 ? 3 : use_cluster(h) ? 2 : use_tile(h) ? 4 : 1;
    if (cluster_size) *cluster_size = h->cluster_ok ? h->csize : 0;
    return ESP_OK;
}

int esp_num_freq(const esp_handle *h, int32_t *nf)
{
    if (!h || !nf) return ESP_EINVAL;
    *nf = h->nf;
    return ESP_OK;
}

int esp_launch_count(const esp_handle *h, int64_t *count)
{
    if (!h || !count) return ESP_EINVAL;
    *count = h->launches;
    return ESP_OK;
}

int esp_begin(esp_handle *h, const esp_schedule *s)
{
    int rc = require(h, true, true);
    if (rc) return rc;
    if (!s) { h->err = "null schedule"; return ESP_EINVAL; }
    if (s->steps_mc < 1 || s->steps_warmup < 0 || s->steps_measure < 0 || (s->pt && s->pt_steps_swap < 1)) {
        h->err = "invalid schedule";
        return ESP_EINVAL;
    }
    const int R = h->R, N = h->N;
    const int nlev = s->lbinerror ? s->num_binning_level : 0;
    if (nlev > 0 && !s->binning_level) { h->err = "binning_level missing"; return ESP_EINVAL; }
    for (int l = 0; l < nlev; ++l)
        if (s->binning_level[l] <= 0 || s->binning_level[l] > 62) { h->err = "binning_level out of range"; return ESP_EINVAL; }
    if ((rc = ensure_levels(h, nlev, s->binning_level))) return rc;
    RunState &u = h->run;
    u = RunState();
    u.s = *s;
    u.levels.assign(s->binning_level, s->binning_level + nlev);
    u.nlev = nlev;
    CK(cudaMemsetAsync(h->d_data, 0, sizeof(double) * 6 * R, h->st));
    CK(cudaMemsetAsync(h->d_pm, 0, sizeof(unsigned long long) * R * h->nf, h->st));
    if (h->obs) {
        CK(cudaMemsetAsync(h->d_obs_data, 0, sizeof(double) * 6 * R, h->st));
        CK(cudaMemsetAsync(h->d_obs_pm, 0, sizeof(unsigned long long) * 2 * R * h->nf, h->st));
    }
    if (h->sc_B) CK(cudaMemsetAsync(h->d_sc_acc, 0, sizeof(double) * 3 * (size_t)R * h->sc_B, h->st));
    if (h->sf_nq) {
        CK(cudaMemsetAsync(h->d_sf_acc, 0, sizeof(double) * 3 * (size_t)R * h->sf_nq, h->st));
        CK(cudaMemsetAsync(h->d_sf_count, 0, sizeof(unsigned long long), h->st));
    }
    CK(cudaMemsetAsync(h->d_rej, 0, sizeof(unsigned long long) * 2 * R, h->st));
    CK(cudaMemsetAsync(h->d_swaps, 0, sizeof(long long) * 2 * R, h->st));
    // a tensor-core wait that gave up is reported by the esp_collect of the
    // run it happened in; a new run starts clean
    if (h->d_tc_err) CK(cudaMemsetAsync(h->d_tc_err, 0, sizeof(int), h->st));
    esp_sweep_opts o;
    o.mcarlo_mode = s->mcarlo_mode; o.tilt_angles_max = s->tilt_angles_max; o.seed = s->seed; o.phase = 0;
    u.e_init.assign(R, 0.0);
    if (!s->pt) {
        // mcarlo.F90:506-521: direct energy, then the warm-up sweeps
        if ((rc = esp_energy(h, u.e_init.data()))) return rc;
        if ((rc = do_sweeps(h, s->steps_warmup * s->steps_measure, h->next_sweep, &o))) return rc;
        h->next_sweep += s->steps_warmup * s->steps_measure;
        if ((rc = fold(h))) return rc;
        u.steps_tot[0] = s->steps_warmup * s->steps_measure * (int64_t)N;
        u.total_units = s->steps_mc;
    } else {
        // pt.F90:524-735: warm-up halved into plain sweeps and swapped sweeps,
        // both rounded up to whole swap intervals
        const int64_t pss = s->pt_steps_swap;
        int64_t sw = ceil_div(s->steps_warmup, 2);
        const int64_t nsw_warm = ceil_div(sw, pss);
        sw = nsw_warm * pss;
        u.total_units = ceil_div(s->steps_mc, pss);
        if ((rc = esp_energy(h, nullptr))) return rc;
        if (sw > 0) {
            if ((rc = do_sweeps(h, sw * s->steps_measure, h->next_sweep, &o))) return rc;
            h->next_sweep += sw * s->steps_measure;
            for (int64_t l = 1; l <= nsw_warm; ++l) {
                if ((rc = do_sweeps(h, pss * s->steps_measure, h->next_sweep, &o))) return rc;
                h->next_sweep += pss * s->steps_measure;
                if ((rc = esp_pt_swap(h, (int)((l + 1) % 2) + 1, h->next_swap++, s->seed))) return rc;
            }
        }
        u.steps_tot[0] = 2 * sw * s->steps_measure * (int64_t)N;
        if ((rc = fold(h))) return rc;
        if ((rc = by_slot(h, h->d_e_run, 1, u.e_init.data()))) return rc;
        CK(cudaMemsetAsync(h->d_swaps, 0, sizeof(long long) * 2 * R, h->st));
    }
    u.active = true;
    return ESP_OK;
}

int esp_advance(esp_handle *h, int64_t n)
{
    int rc = require(h, true, true);
    if (rc) return rc;
    RunState &u = h->run;
    if (!u.active) { h->err = "esp_begin has not been called"; return ESP_ESTATE; }
    if (n < 0) { h->err = "negative step count"; return ESP_EINVAL; }
    const esp_schedule &s = u.s;
    esp_sweep_opts o;
    o.mcarlo_mode = s.mcarlo_mode; o.tilt_angles_max = s.tilt_angles_max; o.seed = s.seed; o.phase = 1;
    if (use_cluster(h)) {
        // spin correlations and the structure factor are measured by their
        // own kernels after a measurement, so each launch then runs one
        // measurement unit
        const int64_t chunk = (h->sc_B || h->sf_nq) ? 1 : kChunk;
        if (!s.pt) {
            // independent temperatures: many measurement units per launch
            for (int64_t done = 0; done < n; done += chunk) {
                const int64_t k = std::min(chunk, n - done);
                if ((rc = cluster_run(h, k, (int)s.steps_measure, h->next_sweep, 1, u.meas_done, &o, 1, u.nlev, false)))
                    return rc;
                h->next_sweep += k * s.steps_measure;
                u.meas_done += k;
                if (h->na == 1) u.const_hits += k;
                if ((h->sc_B || h->sf_nq) && (rc = extra_measure(h, u.meas_done))) return rc;
            }
            u.units_done += n;
        } else {
            for (int64_t k = 0; k < n; ++k) {
                const int64_t l = ++u.units_done;
                for (int64_t done = 0; done < s.pt_steps_swap; done += chunk) {
                    const int64_t m = std::min(chunk, s.pt_steps_swap - done);
                    if ((rc = cluster_run(h, m, (int)s.steps_measure, h->next_sweep, 1, u.meas_done, &o, 1, u.nlev,
                                          true)))
                        return rc;
                    h->next_sweep += m * s.steps_measure;
                    u.meas_done += m;
                    if (h->na == 1) u.const_hits += m;
                    if ((h->sc_B || h->sf_nq) && (rc = extra_measure(h, u.meas_done))) return rc;
                }
                if ((rc = pt_swap_launch(h, (int)((l + 1) % 2) + 1, h->next_swap++, s.seed, l))) return rc;
            }
        }
        return ESP_OK;
    }
    for (int64_t k = 0; k < n; ++k) {
        if (!s.pt) {
            // mcarlo.F90:526-590: steps_measure sweeps, then one measurement
            if ((rc = do_sweeps(h, s.steps_measure, h->next_sweep, &o))) return rc;
            h->next_sweep += s.steps_measure;
            ++u.meas_done;
            if ((rc = measure(h, u.meas_done, u.nlev, false, u.const_hits))) return rc;
        } else {
            // pt.F90:773-907: one swap interval, then pt_swap
            const int64_t l = ++u.units_done;
            for (int64_t mc = 1; mc <= s.pt_steps_swap; ++mc) {
                if ((rc = do_sweeps(h, s.steps_measure, h->next_sweep, &o))) return rc;
                h->next_sweep += s.steps_measure;
                ++u.meas_done;
                if ((rc = measure(h, u.meas_done, u.nlev, true, u.const_hits))) return rc;
            }
            if ((rc = pt_swap_launch(h, (int)((l + 1) % 2) + 1, h->next_swap++, s.seed, l))) return rc;
        }
    }
    if (!s.pt) u.units_done += n;
    return ESP_OK;
}

int esp_collect(esp_handle *h, esp_results *res)
{
    int rc = require(h, true, true);
    if (rc) return rc;
    RunState &u = h->run;
    if (!u.active) { h->err = "esp_begin has not been called"; return ESP_ESTATE; }
    if (!res) { h->err = "null results"; return ESP_EINVAL; }
    if (u.meas_done < 1) { h->err = "no measurement has been made (esp_advance)"; return ESP_ESTATE; }
    if (h->d_tc_err) {
        int flag = 0;
        if ((rc = d2h(h, &flag, h->d_tc_err, sizeof(int)))) return rc;
        if (flag) { h->err = "a tensor-core completion wait of the learned sweep gave up"; return ESP_ETIMEOUT; }
    }
    const int R = h->R, N = h->N, nlev = u.nlev;
    const esp_schedule &s = u.s;
    const int64_t steps_mc = u.meas_done;
    std::vector<double> e_add(R), e_dir(R);
    if ((rc = fold(h))) return rc;
    if ((rc = by_slot(h, h->d_e_run, 1, e_add.data()))) return rc;
    if ((rc = do_energy(h))) return rc;
    if ((rc = by_slot(h, h->d_tmp_e, 1, e_dir.data()))) return rc;
    const double norm = 1.0 / (double)steps_mc;
    std::vector<double> data((size_t)R * 6);
    if ((rc = d2h(h, data.data(), h->d_data, sizeof(double) * 6 * R))) return rc;
    std::vector<unsigned long long> rej((size_t)R * 2);
    if ((rc = d2h(h, rej.data(), h->d_rej, sizeof(unsigned long long) * 2 * R))) return rc;
    res->steps_mc_eff = steps_mc;
    if (res->steps_tot) { res->steps_tot[0] = u.steps_tot[0]; res->steps_tot[1] = steps_mc * s.steps_measure * (int64_t)N; }
    if (res->rejected)
        for (int t = 0; t < 2 * R; ++t) res->rejected[t] = (int64_t)rej[t];
    if (res->energy)
        for (int t = 0; t < R; ++t) {
            res->energy[3 * t] = u.e_init[t]; res->energy[3 * t + 1] = e_add[t]; res->energy[3 * t + 2] = e_dir[t];
        }
    if (res->data)
        for (int i = 0; i < 6 * R; ++i) res->data[i] = data[i] * norm;
    if (res->pm) {
        std::vector<unsigned long long> cnt((size_t)R * h->nf);
        if ((rc = d2h(h, cnt.data(), h->d_pm, sizeof(unsigned long long) * R * h->nf))) return rc;
        const double ncell = (double)(N / h->na);
        for (int t = 0; t < R; ++t) {
            if (h->na == 1) cnt[(size_t)t * h->nf + h->nf - 1] += (unsigned long long)(u.const_hits * (long long)ncell);
            // each hit adds 1/d_m = 100 (get_quant.F90:487); normalised by
            // steps_mc * num_supercell (mcarlo.F90:715)
            for (int f = 0; f < h->nf; ++f)
                res->pm[(size_t)t * h->nf + f] = (double)cnt[(size_t)t * h->nf + f] * (1.0 / 0.01) * norm / ncell;
        }
    }
    if (res->binning && nlev > 0) {
        std::vector<double> ls((size_t)R * nlev * 2), bn((size_t)R * nlev * 2);
        if ((rc = d2h(h, ls.data(), h->d_lsum, sizeof(double) * ls.size()))) return rc;
        if ((rc = d2h(h, bn.data(), h->d_bin, sizeof(double) * bn.size()))) return rc;
        // mcarlo.F90:635-656 / pt.F90:914-936
        for (int t = 0; t < R; ++t)
            for (int l = 0; l < nlev; ++l) {
                const double blk = (double)(1LL << u.levels[l]);
                const double m_l = (double)(steps_mc / (1LL << u.levels[l]));
                for (int c = 0; c < 2; ++c) {
                    const size_t k = ((size_t)t * nlev + l) * 2 + c;
                    const double tot = c == 0 ? data[6 * t] / (double)N : data[6 * t + 3];
                    double v = (tot - ls[k]) / blk / m_l;
                    double b = bn[k] / m_l;
                    b = (b - v * v) / (m_l - 1.0);
                    if (s.pt) b = b / (double)N;
                    res->binning[k] = b;
                }
            }
    }
    if (res->num_swaps || res->map) {
        std::vector<long long> sw((size_t)R * 2);
        if ((rc = d2h(h, sw.data(), h->d_swaps, sizeof(long long) * 2 * R))) return rc;
        if (res->num_swaps) for (int i = 0; i < 2 * R; ++i) res->num_swaps[i] = sw[i];
        if (res->map) {
            std::vector<int32_t> ra;
            if ((rc = get_repl_at(h, ra))) return rc;
            for (int t = 0; t < R; ++t) res->map[t] = ra[t] + 1;
        }
    }
    return ESP_OK;
}

int esp_set_observables(esp_handle *h, int32_t flags, const double *orderparam_axes, const int32_t *staggered_coeff)
{
    if (!h) return ESP_EINVAL;
    if (!h->have_tables) { h->err = "upload the tables before choosing the optional measurements"; return ESP_ESTATE; }
    if (flags & ~(ESP_OBS_ORDER_PARAMETER | ESP_OBS_STAGGERED)) { h->err = "unknown measurement flag"; return ESP_EINVAL; }
    if ((flags & ESP_OBS_ORDER_PARAMETER) && !orderparam_axes) { h->err = "order-parameter axes missing"; return ESP_EINVAL; }
    if ((flags & ESP_OBS_STAGGERED) && !staggered_coeff) { h->err = "staggered coefficients missing"; return ESP_EINVAL; }
    std::vector<float4> atom((size_t)h->na);
    for (int at = 0; at < h->na; ++at) {
        float4 w = make_float4(0.f, 0.f, 0.f, 0.f);
        if (flags & ESP_OBS_ORDER_PARAMETER) {
            const double *ax = orderparam_axes + 3 * at;
            if (!std::isfinite(ax[0]) || !std::isfinite(ax[1]) || !std::isfinite(ax[2])) {
                h->err = "order-parameter axes must be finite";
                return ESP_EINVAL;
            }
            w.x = (float)ax[0]; w.y = (float)ax[1]; w.z = (float)ax[2];
        }
        if (flags & ESP_OBS_STAGGERED) {
            if (staggered_coeff[at] != 1 && staggered_coeff[at] != -1) {
                h->err = "staggered_m_coeff must be +1 or -1";
                return ESP_EINVAL;
            }
            w.w = (float)staggered_coeff[at];
        }
        atom[at] = w;
    }
    int rc = fold(h);
    if (rc) return rc;
    CK(cudaStreamSynchronize(h->st));
    free_obs(h);
    if (flags) {
        CK(dalloc(&h->d_obs_atom, (size_t)h->na));
        CK(dalloc(&h->d_obs_rep, (size_t)h->R * 4));
        CK(dalloc(&h->d_obs_data, (size_t)h->R * 6));
        CK(dalloc(&h->d_obs_pm, (size_t)h->R * 2 * h->nf));
        if ((rc = h2d(h, h->d_obs_atom, atom.data(), sizeof(float4) * atom.size()))) return rc;
        CK(cudaMemsetAsync(h->d_obs_data, 0, sizeof(double) * 6 * h->R, h->st));
        CK(cudaMemsetAsync(h->d_obs_pm, 0, sizeof(unsigned long long) * 2 * h->R * h->nf, h->st));
        CK(cudaMemsetAsync(h->d_obs_rep, 0, sizeof(double) * 4 * h->R, h->st));
    }
    h->obs = flags;
    // the cluster kernel keeps two more histograms in shared memory: keep the
    // geometry if it still fits, else take the best one that does
    if (h->cluster_ok) {
        const std::vector<ClusterGeom> c = cluster_candidates(h);
        bool same = false;
        for (const ClusterGeom &g : c) same = same || (g.cs == h->csize && g.nt == h->cthreads && g.S == h->csites);
        if (same) rc = cluster_geometry(h, h->csize, h->cthreads, h->csites);
        else if (!c.empty()) rc = cluster_geometry(h, c[0].cs, c[0].nt, c[0].S);
        else h->cluster_ok = false;
        if (rc) return rc;
    }
    CK(cudaStreamSynchronize(h->st));
    return ESP_OK;
}

int esp_collect_observables(esp_handle *h, esp_obs_results *res)
{
    int rc = require(h, true, true);
    if (rc) return rc;
    RunState &u = h->run;
    if (!u.active) { h->err = "esp_begin has not been called"; return ESP_ESTATE; }
    if (!res) { h->err = "null results"; return ESP_EINVAL; }
    if (!h->obs) { h->err = "no optional measurement was chosen (esp_set_observables)"; return ESP_ESTATE; }
    if (u.meas_done < 1) { h->err = "no measurement has been made (esp_advance)"; return ESP_ESTATE; }
    if ((rc = fold(h))) return rc;
    const int R = h->R, N = h->N, nlev = u.nlev, nf = h->nf;
    const int64_t steps_mc = u.meas_done;
    const double norm = 1.0 / (double)steps_mc;
    std::vector<double> data((size_t)R * 6);
    if ((rc = d2h(h, data.data(), h->d_obs_data, sizeof(double) * data.size()))) return rc;
    // mcarlo.F90:713-715 / pt.F90:995-1000
    if (res->data)
        for (size_t i = 0; i < data.size(); ++i) res->data[i] = data[i] * norm;
    if (res->pm_op || res->pm_sm) {
        std::vector<unsigned long long> cnt((size_t)R * 2 * nf);
        if ((rc = d2h(h, cnt.data(), h->d_obs_pm, sizeof(unsigned long long) * cnt.size()))) return rc;
        const double ncell = (double)(N / h->na);
        for (int t = 0; t < R; ++t)
            for (int f = 0; f < nf; ++f) {
                const size_t o = (size_t)t * nf + f;
                if (res->pm_op) res->pm_op[o] = (double)cnt[((size_t)t * 2) * nf + f] * (1.0 / 0.01) * norm / ncell;
                if (res->pm_sm) res->pm_sm[o] = (double)cnt[((size_t)t * 2 + 1) * nf + f] * (1.0 / 0.01) * norm / ncell;
            }
    }
    if (res->binning && nlev > 0) {
        std::vector<double> ls((size_t)R * nlev * 2), bn((size_t)R * nlev * 2);
        if ((rc = d2h(h, ls.data(), h->d_obs_lsum, sizeof(double) * ls.size()))) return rc;
        if ((rc = d2h(h, bn.data(), h->d_obs_bin, sizeof(double) * bn.size()))) return rc;
        // mcarlo.F90:640-656 / pt.F90:918-936 for the |OP| and |SM| rows
        for (int t = 0; t < R; ++t)
            for (int l = 0; l < nlev; ++l) {
                const double blk = (double)(1LL << u.levels[l]);
                const double m_l = (double)(steps_mc / (1LL << u.levels[l]));
                for (int c = 0; c < 2; ++c) {
                    const size_t k = ((size_t)t * nlev + l) * 2 + c;
                    const double tot = data[6 * t + 3 * c];
                    double v = (tot - ls[k]) / blk / m_l;
                    double b = bn[k] / m_l;
                    b = (b - v * v) / (m_l - 1.0);
                    if (u.s.pt) b = b / (double)N;
                    res->binning[k] = b;
                }
            }
    }
    return ESP_OK;
}

int esp_set_spin_correlation(esp_handle *h, int32_t num_shells, int32_t num_species, int32_t nbors_max,
                             const int32_t *kind_atoms, const int32_t *shell_num_nbors, const int32_t *shell_nbors,
                             const int32_t *shell_num_nbors_kind)
{
    if (!h) return ESP_EINVAL;
    if (!h->have_tables) { h->err = "upload the tables before the spin-correlation shells"; return ESP_ESTATE; }
    if (num_shells < 0 || num_species < 1 || nbors_max < 0) { h->err = "invalid shell dimensions"; return ESP_EINVAL; }
    if (num_shells > 0 && (!kind_atoms || !shell_num_nbors || (nbors_max > 0 && !shell_nbors) || !shell_num_nbors_kind)) {
        h->err = "shell tables missing";
        return ESP_EINVAL;
    }
    const int N = h->N, S = num_shells, nsp = num_species;
    const long long B = (long long)S * nsp * nsp;
    if (B > 4096) { h->err = "more than 4096 spin-correlation bins (shells x species^2)"; return ESP_EINVAL; }
    // per permuted site: entries (neighbour, weight) grouped by bin
    // (shell, species of the site, species of the neighbour), each group in
    // the order of shell_nbors_matrix
    std::vector<std::vector<std::pair<int, std::pair<int, float>>>> lists;
    if (S > 0) {
        for (int i = 0; i < N; ++i)
            if (kind_atoms[i] < 1 || kind_atoms[i] > nsp) { h->err = "kind_atoms out of range"; return ESP_EINVAL; }
        lists.resize(N);
        for (int p = 0; p < N; ++p) {
            const int i = h->prep.perm[p];
            const int a = kind_atoms[i] - 1;
            auto &lst = lists[p];
            for (int sh = 0; sh < S; ++sh) {
                const int nn = shell_num_nbors[(size_t)i * S + sh];
                if (nn < 0 || nn > nbors_max) { h->err = "shell_num_nbors_matrix out of range"; return ESP_EINVAL; }
                for (int k = 0; k < nn; ++k) {
                    const int j = shell_nbors[((size_t)k * N + i) * S + sh] - 1;
                    if (j < 0 || j >= N) { h->err = "shell_nbors_matrix out of range"; return ESP_EINVAL; }
                    const int b = kind_atoms[j] - 1;
                    const int c = shell_num_nbors_kind[((size_t)b * nsp + a) * S + sh];
                    const int bin = (sh * nsp + a) * nsp + b;
                    // get_quant.F90:525-530: 1 / (shell_num_nbors_kind m_i m_j)
                    const double den = (double)c * h->mag_host[i] * h->mag_host[j];
                    lst.push_back({bin, {h->prep.inv[j], (float)(1.0 / den)}});
                }
            }
            std::stable_sort(lst.begin(), lst.end(), [](const auto &x, const auto &y) { return x.first < y.first; });
        }
    }
    int rc = fold(h);
    if (rc) return rc;
    CK(cudaStreamSynchronize(h->st));
    free_sc(h);
    if (S == 0) return ESP_OK;
    size_t maxe = 1;
    for (const auto &l : lists) maxe = std::max(maxe, l.size());
    std::vector<int32_t> off((size_t)(B + 1) * N), nb(maxe * N, 0);
    std::vector<float> w(maxe * N, 0.f);
    for (int p = 0; p < N; ++p) {
        const auto &l = lists[p];
        size_t e = 0;
        for (long long b = 0; b <= B; ++b) {
            while (e < l.size() && l[e].first < b) ++e;
            off[(size_t)b * N + p] = (int32_t)e;
        }
        for (size_t q = 0; q < l.size(); ++q) {
            nb[q * N + p] = l[q].second.first;
            w[q * N + p] = l[q].second.second;
        }
    }
    const int npass = (int)((B + 1) / 2);
    h->sc_blocks = std::max(1, std::min(h->e_blocks, 4 * h->num_sms));
    if (h->sc_blocks * 256LL < h->R) h->sc_blocks = (h->R + 255) / 256;
    CK(dalloc(&h->d_sc_off, off.size()));
    CK(dalloc(&h->d_sc_nb, nb.size()));
    CK(dalloc(&h->d_sc_w, w.size()));
    CK(dalloc(&h->d_sc_scratch, (size_t)npass * h->sc_blocks * h->R * 4));
    CK(dalloc(&h->d_sc_out, (size_t)npass * h->R * 4));
    CK(dalloc(&h->d_sc_acc, (size_t)h->R * B * 3));
    if ((rc = h2d(h, h->d_sc_off, off.data(), sizeof(int32_t) * off.size()))) return rc;
    if ((rc = h2d(h, h->d_sc_nb, nb.data(), sizeof(int32_t) * nb.size()))) return rc;
    if ((rc = h2d(h, h->d_sc_w, w.data(), sizeof(float) * w.size()))) return rc;
    CK(cudaMemsetAsync(h->d_sc_acc, 0, sizeof(double) * 3 * (size_t)h->R * B, h->st));
    CK(cudaStreamSynchronize(h->st));
    h->sc_B = (int)B; h->sc_S = S; h->sc_nsp = nsp;
    return ESP_OK;
}

int esp_collect_spin_correlation(esp_handle *h, double *spincorr, double *spincorr_abs, double *spincorr_tot_abs)
{
    int rc = require(h, true, true);
    if (rc) return rc;
    RunState &u = h->run;
    if (!u.active) { h->err = "esp_begin has not been called"; return ESP_ESTATE; }
    if (!h->sc_B) { h->err = "no spin-correlation shells were set (esp_set_spin_correlation)"; return ESP_ESTATE; }
    if (u.meas_done < 1) { h->err = "no measurement has been made (esp_advance)"; return ESP_ESTATE; }
    if ((rc = fold(h))) return rc;
    const size_t B = (size_t)h->sc_B, R = (size_t)h->R;
    std::vector<double> acc(R * B * 3);
    if ((rc = d2h(h, acc.data(), h->d_sc_acc, sizeof(double) * acc.size()))) return rc;
    // global_spincorr * normalize / N (mcarlo.F90:717-723, pt.F90:1003-1009)
    const double normalize = 1.0 / (double)u.meas_done;
    double *outs[3] = {spincorr, spincorr_abs, spincorr_tot_abs};
    for (int c = 0; c < 3; ++c)
        if (outs[c])
            for (size_t k = 0; k < R * B; ++k) outs[c][k] = acc[k * 3 + c] * normalize / (double)h->N;
    return ESP_OK;
}

int esp_set_structure_factor(esp_handle *h, int32_t nq, const double *qpts, const double *polar,
                             int32_t steps_measure, const double *real_lattice, const double *pos)
{
    if (!h) return ESP_EINVAL;
    if (!h->have_tables) { h->err = "upload the tables before the structure factor"; return ESP_ESTATE; }
    if (nq < 0 || (nq > 0 && (!qpts || !polar || !real_lattice || !pos || steps_measure < 1))) {
        h->err = "invalid structure-factor arguments";
        return ESP_EINVAL;
    }
    if ((long long)nq * h->R > (1LL << 31) / 8) { h->err = "too many q-points x replicas"; return ESP_EINVAL; }
    const int N = h->N;
    std::vector<int4> sn;
    std::vector<float4> sf_f, qf, qc;
    std::vector<uint4> qfix;
    double pnorm = 1.0;
    if (nq > 0) {
        // a_j = real_lattice(j, :), Fortran column-major
        double A[3][3];
        for (int j = 0; j < 3; ++j)
            for (int i = 0; i < 3; ++i) A[j][i] = real_lattice[j + 3 * i];
        // pos = sum_j u_j a_j: u = M pos with M the inverse of the transpose of A
        const double det = A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) -
                           A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
                           A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
        if (!(std::fabs(det) > 1e-12)) { h->err = "singular real_lattice"; return ESP_EINVAL; }
        double M[3][3];   // M[j][i]: u_j = sum_i M[j][i] pos_i, rows of the reciprocal lattice / 2 pi
        M[0][0] = (A[1][1] * A[2][2] - A[1][2] * A[2][1]) / det;
        M[0][1] = (A[1][2] * A[2][0] - A[1][0] * A[2][2]) / det;
        M[0][2] = (A[1][0] * A[2][1] - A[1][1] * A[2][0]) / det;
        M[1][0] = (A[2][1] * A[0][2] - A[2][2] * A[0][1]) / det;
        M[1][1] = (A[2][2] * A[0][0] - A[2][0] * A[0][2]) / det;
        M[1][2] = (A[2][0] * A[0][1] - A[2][1] * A[0][0]) / det;
        M[2][0] = (A[0][1] * A[1][2] - A[0][2] * A[1][1]) / det;
        M[2][1] = (A[0][2] * A[1][0] - A[0][0] * A[1][2]) / det;
        M[2][2] = (A[0][0] * A[1][1] - A[0][1] * A[1][0]) / det;
        sn.resize(N); sf_f.resize(N);
        for (int i = 0; i < N; ++i) {
            double u[3], n[3];
            for (int j = 0; j < 3; ++j) {
                u[j] = M[j][0] * pos[3 * i] + M[j][1] * pos[3 * i + 1] + M[j][2] * pos[3 * i + 2];
                n[j] = std::floor(u[j]);
                if (std::fabs(n[j]) > 1e9) { h->err = "site position too far from the origin"; return ESP_EINVAL; }
            }
            sn[i] = make_int4((int)n[0], (int)n[1], (int)n[2], 0);
            sf_f[i] = make_float4((float)(u[0] - n[0]), (float)(u[1] - n[1]), (float)(u[2] - n[2]), 0.f);
        }
        qf.resize(nq); qc.resize(nq); qfix.resize(nq);
        const double two32 = 4294967296.0, twopi = 6.283185307179586476925286766559;
        for (int k = 0; k < nq; ++k) {
            const double *q = qpts + 3 * k;
            double f[3];
            uint32_t fx[3];
            for (int j = 0; j < 3; ++j) {
                f[j] = (q[0] * A[j][0] + q[1] * A[j][1] + q[2] * A[j][2]) / twopi;
                const double fr = f[j] - std::floor(f[j]);
                fx[j] = (uint32_t)(unsigned long long)std::llround(fr * two32);
            }
            qfix[k] = make_uint4(fx[0], fx[1], fx[2], 0u);
            qf[k] = make_float4((float)f[0], (float)f[1], (float)f[2], 0.f);
            const bool zero = q[0] == 0.0 && q[1] == 0.0 && q[2] == 0.0;
            qc[k] = make_float4((float)q[0], (float)q[1], (float)q[2], zero ? 1.f : 0.f);
        }
        pnorm = std::sqrt(polar[0] * polar[0] + polar[1] * polar[1] + polar[2] * polar[2]);
        if (!(pnorm > 0.0)) { h->err = "sfactor_polar must not be zero"; return ESP_EINVAL; }
    }
    int rc = fold(h);
    if (rc) return rc;
    CK(cudaStreamSynchronize(h->st));
    free_sf(h);
    if (nq == 0) return ESP_OK;
    CK(dalloc(&h->d_sf_n, (size_t)N));
    CK(dalloc(&h->d_sf_f, (size_t)N));
    CK(dalloc(&h->d_sf_qfix, (size_t)nq));
    CK(dalloc(&h->d_sf_qf, (size_t)nq));
    CK(dalloc(&h->d_sf_qc, (size_t)nq));
    CK(dalloc(&h->d_sf_fq, (size_t)nq * h->R * 6));
    CK(dalloc(&h->d_sf_acc, (size_t)nq * h->R * 3));
    CK(dalloc(&h->d_sf_count, 1));
    if ((rc = h2d(h, h->d_sf_n, sn.data(), sizeof(int4) * N))) return rc;
    if ((rc = h2d(h, h->d_sf_f, sf_f.data(), sizeof(float4) * N))) return rc;
    if ((rc = h2d(h, h->d_sf_qfix, qfix.data(), sizeof(uint4) * nq))) return rc;
    if ((rc = h2d(h, h->d_sf_qf, qf.data(), sizeof(float4) * nq))) return rc;
    if ((rc = h2d(h, h->d_sf_qc, qc.data(), sizeof(float4) * nq))) return rc;
    CK(cudaMemsetAsync(h->d_sf_acc, 0, sizeof(double) * 3 * (size_t)nq * h->R, h->st));
    CK(cudaMemsetAsync(h->d_sf_count, 0, sizeof(unsigned long long), h->st));
    CK(cudaStreamSynchronize(h->st));
    h->sf_nq = nq; h->sf_every = steps_measure;
    for (int c = 0; c < 3; ++c) h->sf_p[c] = polar[c];
    h->sf_pnorm = pnorm;
    return ESP_OK;
}

int esp_collect_structure_factor(esp_handle *h, double *sf, int64_t *num_measured)
{
    int rc = require(h, true, true);
    if (rc) return rc;
    RunState &u = h->run;
    if (!u.active) { h->err = "esp_begin has not been called"; return ESP_ESTATE; }
    if (!h->sf_nq) { h->err = "no structure factor was set (esp_set_structure_factor)"; return ESP_ESTATE; }
    if ((rc = fold(h))) return rc;
    unsigned long long cnt = 0;
    if ((rc = d2h(h, &cnt, h->d_sf_count, sizeof(cnt)))) return rc;
    if (num_measured) *num_measured = (int64_t)cnt;
    if (sf) {
        const size_t n = (size_t)h->R * h->sf_nq * 3;
        if ((rc = d2h(h, sf, h->d_sf_acc, sizeof(double) * n))) return rc;
        // global_sfactor_matrix / N / num_sfsteps_tot (mcarlo.F90:821-822)
        for (size_t k = 0; k < n; ++k) sf[k] = cnt ? sf[k] / (double)h->N / (double)cnt : 0.0;
    }
    return ESP_OK;
}

int esp_run(esp_handle *h, const esp_schedule *s, esp_results *res)
{
    int rc = esp_begin(h, s);
    if (rc) return rc;
    if ((rc = esp_advance(h, h->run.total_units))) return rc;
    return esp_collect(h, res);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Learned proposal: network storage, training set, training passes.
// ---------------------------------------------------------------------------
namespace {

// logical parameter order: W1[128][12] b1[128] W2[128][128] b2[128] W3[20][128] b3[20]
void lp_logical_to_padded(const float *in, std::vector<float> &p)
{
    p.assign(kPadParams, 0.f);
    size_t o = 0;
    for (int n = 0; n < kMlpHid; ++n)
        for (int k = 0; k < kMlpIn; ++k) p[kPadW1 + n * kMlpInPad + k] = in[o++];
    for (int n = 0; n < kMlpHid; ++n) p[kPadB1 + n] = in[o++];
    for (int i = 0; i < kMlpHid * kMlpHid; ++i) p[kPadW2 + i] = in[o++];
    for (int n = 0; n < kMlpHid; ++n) p[kPadB2 + n] = in[o++];
    for (int n = 0; n < kMlpOut; ++n)
        for (int k = 0; k < kMlpHid; ++k) p[kPadW3 + n * kMlpHid + k] = in[o++];
    for (int n = 0; n < kMlpOut; ++n) p[kPadB3 + n] = in[o++];
}

void lp_padded_to_logical(const std::vector<float> &p, float *out)
{
    size_t o = 0;
    for (int n = 0; n < kMlpHid; ++n)
        for (int k = 0; k < kMlpIn; ++k) out[o++] = p[kPadW1 + n * kMlpInPad + k];
    for (int n = 0; n < kMlpHid; ++n) out[o++] = p[kPadB1 + n];
    for (int i = 0; i < kMlpHid * kMlpHid; ++i) out[o++] = p[kPadW2 + i];
    for (int n = 0; n < kMlpHid; ++n) out[o++] = p[kPadB2 + n];
    for (int n = 0; n < kMlpOut; ++n)
        for (int k = 0; k < kMlpHid; ++k) out[o++] = p[kPadW3 + n * kMlpHid + k];
    for (int n = 0; n < kMlpOut; ++n) out[o++] = p[kPadB3 + n];
}

int lp_alloc_net(esp_handle *h)
{
    if (h->d_lp_p) return ESP_OK;
    CK(dalloc(&h->d_lp_p, kPadParams));
    CK(dalloc(&h->d_lp_g, kPadParams));
    CK(dalloc(&h->d_lp_m, kPadParams));
    CK(dalloc(&h->d_lp_v, kPadParams));
    CK(dalloc(&h->d_lp_w1, kMlpHid * kMlpInPad));
    CK(dalloc(&h->d_lp_w2, kMlpHid * kMlpHid));
    CK(dalloc(&h->d_lp_w3, kMlpOutPad * kMlpHid));
    return ESP_OK;
}

// Upload padded fp32 parameters, reset Adam, refresh the bf16 copies.
int lp_upload(esp_handle *h, const std::vector<float> &p)
{
    int rc = lp_alloc_net(h);
    if (rc) return rc;
    CK(cudaMemcpyAsync(h->d_lp_p, p.data(), sizeof(float) * kPadParams, cudaMemcpyHostToDevice, h->st));
    CK(cudaMemsetAsync(h->d_lp_m, 0, sizeof(float) * kPadParams, h->st));
    CK(cudaMemsetAsync(h->d_lp_v, 0, sizeof(float) * kPadParams, h->st));
    CK(launch_lp_to_bf16(h->d_lp_p, h->d_lp_w1, h->d_lp_w2, h->d_lp_w3, h->st));
    h->launches++;
    CK(cudaStreamSynchronize(h->st));
    h->lp_adam_t = 0;
    h->lp_weights = true;
    return ESP_OK;
}

int lp_ensure_batch(esp_handle *h, int B)
{
    if (B <= h->lp_bcap) return ESP_OK;
    free_lp_batch(h);
    const size_t b = (size_t)B;
    CK(dalloc(&h->d_lp_xb, b * kMlpInPad));
    CK(dalloc(&h->d_lp_h1, b * kMlpHid));
    CK(dalloc(&h->d_lp_h2, b * kMlpHid));
    CK(dalloc(&h->d_lp_do, b * kMlpOutPad));
    CK(dalloc(&h->d_lp_dz2, b * kMlpHid));
    CK(dalloc(&h->d_lp_dz1, b * kMlpHid));
    CK(dalloc(&h->d_lp_tb, b * 4));
    CK(dalloc(&h->d_lp_o, b * kMlpOutPad));
    h->lp_bcap = B;
    return ESP_OK;
}

int lp_ensure_loss(esp_handle *h, long long n)
{
    if (n <= h->lp_loss_cap) return ESP_OK;
    dfree(h->d_lp_loss);
    CK(dalloc(&h->d_lp_loss, (size_t)n));
    h->lp_loss_cap = n;
    return ESP_OK;
}

// ESP_ETIMEOUT when a tensor-core completion wait of the tcgen05 engine gave up
// since the flag was last cleared.
int lp_tc_status(esp_handle *h, const char *what)
{
    if (h->lp_engine != 1 || !h->d_tc_err) return ESP_OK;
    int flag = 0;
    int rc = d2h(h, &flag, h->d_tc_err, sizeof(int));
    if (rc) return rc;
    if (flag) { h->err = std::string(what) + ": a tensor-core completion wait gave up"; return ESP_ETIMEOUT; }
    return ESP_OK;
}

// Forward and backward pass over the B rows in the batch buffers, the first
// n_real of which are samples: loss (mean -log q over those) into *d_loss,
// gradients into d_lp_g (padded layout).
int lp_pass(esp_handle *h, int B, int n_real, double *d_loss)
{
    cudaStream_t st = h->st;
    const float *P = h->d_lp_p;
    float *G = h->d_lp_g;
    GemmArgs g;
    auto reset = [&]() { std::memset(&g, 0, sizeof(g)); };
    // the network's engine also runs the training GEMMs: warp-level mma.sync
    // tiles, or tcgen05 with tensor-memory accumulators
    auto gemm = [&](bool ta, bool tb) -> cudaError_t {
        if (h->lp_engine == 1) return launch_gemm_tc(g, ta, tb, h->num_sms, h->d_lp_gwork, h->d_tc_err, st);
        return launch_gemm(g, ta, tb, st);
    };
    // H1 = relu(X W1^T + b1)
    reset(); g.A = h->d_lp_xb; g.lda = kMlpInPad; g.B = h->d_lp_w1; g.ldb = kMlpInPad;
    g.M = B; g.N = kMlpHid; g.K = kMlpInPad; g.Cb = h->d_lp_h1; g.ldcb = kMlpHid; g.bias = P + kPadB1; g.relu = 1;
    CK(gemm(false, false));
    // H2 = relu(H1 W2^T + b2)
    reset(); g.A = h->d_lp_h1; g.lda = kMlpHid; g.B = h->d_lp_w2; g.ldb = kMlpHid;
    g.M = B; g.N = kMlpHid; g.K = kMlpHid; g.Cb = h->d_lp_h2; g.ldcb = kMlpHid; g.bias = P + kPadB2; g.relu = 1;
    CK(gemm(false, false));
    // O = H2 W3^T + b3
    reset(); g.A = h->d_lp_h2; g.lda = kMlpHid; g.B = h->d_lp_w3; g.ldb = kMlpHid;
    g.M = B; g.N = kMlpOutPad; g.K = kMlpHid; g.C = h->d_lp_o; g.ldc = kMlpOutPad; g.bias = P + kPadB3;
    CK(gemm(false, false));
    // dO
    CK(launch_lp_head(h->d_lp_o, h->d_lp_tb, n_real, B, 1.f / (float)n_real, h->d_lp_do, d_loss, st));
    // dW3 = dO^T H2, db3
    reset(); g.A = h->d_lp_do; g.lda = kMlpOutPad; g.B = h->d_lp_h2; g.ldb = kMlpHid;
    g.M = kMlpOutPad; g.N = kMlpHid; g.K = B; g.C = G + kPadW3; g.ldc = kMlpHid;
    CK(gemm(true, true));
    CK(launch_colsum(h->d_lp_do, B, kMlpOutPad, kMlpOutPad, G + kPadB3, st));
    // dZ2 = (dO W3) . [H2 > 0]
    reset(); g.A = h->d_lp_do; g.lda = kMlpOutPad; g.B = h->d_lp_w3; g.ldb = kMlpHid;
    g.M = B; g.N = kMlpHid; g.K = kMlpOutPad; g.Cb = h->d_lp_dz2; g.ldcb = kMlpHid; g.mask = h->d_lp_h2; g.ldm = kMlpHid;
    CK(gemm(false, true));
    // dW2 = dZ2^T H1, db2
    reset(); g.A = h->d_lp_dz2; g.lda = kMlpHid; g.B = h->d_lp_h1; g.ldb = kMlpHid;
    g.M = kMlpHid; g.N = kMlpHid; g.K = B; g.C = G + kPadW2; g.ldc = kMlpHid;
    CK(gemm(true, true));
    CK(launch_colsum(h->d_lp_dz2, B, kMlpHid, kMlpHid, G + kPadB2, st));
    // dZ1 = (dZ2 W2) . [H1 > 0]
    reset(); g.A = h->d_lp_dz2; g.lda = kMlpHid; g.B = h->d_lp_w2; g.ldb = kMlpHid;
    g.M = B; g.N = kMlpHid; g.K = kMlpHid; g.Cb = h->d_lp_dz1; g.ldcb = kMlpHid; g.mask = h->d_lp_h1; g.ldm = kMlpHid;
    CK(gemm(false, true));
    // dW1 = dZ1^T X, db1
    reset(); g.A = h->d_lp_dz1; g.lda = kMlpHid; g.B = h->d_lp_xb; g.ldb = kMlpInPad;
    g.M = kMlpHid; g.N = kMlpInPad; g.K = B; g.C = G + kPadW1; g.ldc = kMlpInPad;
    CK(gemm(true, true));
    CK(launch_colsum(h->d_lp_dz1, B, kMlpHid, kMlpHid, G + kPadB1, st));
    h->launches += 13;
    return ESP_OK;
}

void bf16_rows(const float *f, int64_t n, std::vector<__nv_bfloat16> &x)
{
    x.assign((size_t)n * kMlpInPad, __float2bfloat16_rn(0.f));
    for (int64_t i = 0; i < n; ++i)
        for (int k = 0; k < kMlpIn; ++k) x[(size_t)i * kMlpInPad + k] = __float2bfloat16_rn(f[(size_t)i * kMlpIn + k]);
}

int64_t round8(int64_t n) { return (n + 7) & ~(int64_t)7; }

}  // namespace

extern "C" {

int esp_lp_num_params(void) { return kLpParams; }

int esp_lp_set_weights(esp_handle *h, const float *params)
{
    if (!h || !params) return ESP_EINVAL;
    for (int i = 0; i < kLpParams; ++i)
        if (!std::isfinite(params[i])) { h->err = "non-finite network parameter"; return ESP_EINVAL; }
    std::vector<float> p;
    lp_logical_to_padded(params, p);
    return lp_upload(h, p);
}

int esp_lp_get_weights(esp_handle *h, float *params)
{
    if (!h || !params) return ESP_EINVAL;
    if (!h->lp_weights) { h->err = "no network weights (esp_lp_init_weights / esp_lp_set_weights)"; return ESP_ESTATE; }
    std::vector<float> p(kPadParams);
    int rc = d2h(h, p.data(), h->d_lp_p, sizeof(float) * kPadParams);
    if (rc) return rc;
    lp_padded_to_logical(p, params);
    return ESP_OK;
}

int esp_lp_init_weights(esp_handle *h, uint64_t seed)
{
    if (!h) return ESP_EINVAL;
    // splitmix64 uniforms: He-uniform hidden layers, a small output layer so
    // that the initial proposal is close to the Heisenberg conditional
    uint64_t state = seed ^ 0x6A09E667F3BCC909ull;
    auto uni = [&]() {
        uint64_t z = (state += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
    };
    std::vector<float> l(kLpParams, 0.f);
    size_t o = 0;
    const double a1 = std::sqrt(6.0 / kMlpIn), a2 = std::sqrt(6.0 / kMlpHid), a3 = 0.01 / std::sqrt((double)kMlpHid);
    for (int i = 0; i < kMlpHid * kMlpIn; ++i) l[o++] = (float)(a1 * uni());
    o += kMlpHid;
    for (int i = 0; i < kMlpHid * kMlpHid; ++i) l[o++] = (float)(a2 * uni());
    o += kMlpHid;
    for (int i = 0; i < kMlpOut * kMlpHid; ++i) l[o++] = (float)(a3 * uni());
    std::vector<float> p;
    lp_logical_to_padded(l.data(), p);
    return lp_upload(h, p);
}

int esp_lp_reserve(esp_handle *h, int64_t capacity)
{
    if (!h || capacity < 0) return ESP_EINVAL;
    CK(cudaStreamSynchronize(h->st));
    dfree(h->d_lp_x); dfree(h->d_lp_t);
    h->lp_cap = 0; h->lp_n = 0;
    if (capacity == 0) return ESP_OK;
    CK(dalloc(&h->d_lp_x, (size_t)capacity * kMlpInPad));
    CK(dalloc(&h->d_lp_t, (size_t)capacity * 4));
    h->lp_cap = capacity;
    return ESP_OK;
}

int esp_lp_collect(esp_handle *h, int32_t colour, int64_t *rows)
{
    int rc = require(h, true, true);
    if (rc) return rc;
    if (colour < 0 || colour >= h->prep.num_colours) { h->err = "bad colour"; return ESP_EINVAL; }
    if (h->lp_cap == 0) { h->err = "no training-set storage (esp_lp_reserve)"; return ESP_ESTATE; }
    if ((rc = arrays_current(h))) return rc;
    esp_sweep_opts o{};
    LpCollectArgs c;
    c.s = sweep_args(h, colour, 0, &o);
    c.axis = h->hsi ? h->d_lp_axis : nullptr;
    c.x = h->d_lp_x; c.t = h->d_lp_t;
    c.first = h->lp_n;
    c.count = std::min((long long)c.s.n_c * h->R, h->lp_cap - h->lp_n);
    CK(launch_lp_collect(c, h->prep.has_b, h->prep.has_d, h->max_blocks, h->st));
    h->launches++;
    h->lp_n += c.count;
    if (rows) *rows = h->lp_n;
    return ESP_OK;
}

int esp_lp_get_data(esp_handle *h, int64_t first, int64_t n, float *features, float *targets)
{
    if (!h || first < 0 || n < 0 || first + n > h->lp_n) return ESP_EINVAL;
    if (n == 0) return ESP_OK;
    std::vector<__nv_bfloat16> x((size_t)n * kMlpInPad);
    std::vector<float> t((size_t)n * 4);
    int rc = d2h(h, x.data(), h->d_lp_x + (size_t)first * kMlpInPad, sizeof(__nv_bfloat16) * x.size());
    if (rc) return rc;
    if ((rc = d2h(h, t.data(), h->d_lp_t + (size_t)first * 4, sizeof(float) * t.size()))) return rc;
    for (int64_t i = 0; i < n; ++i) {
        if (features)
            for (int k = 0; k < kMlpIn; ++k) features[i * kMlpIn + k] = __bfloat162float(x[(size_t)i * kMlpInPad + k]);
        if (targets)
            for (int k = 0; k < 4; ++k) targets[i * 4 + k] = t[(size_t)i * 4 + k];
    }
    return ESP_OK;
}

int esp_lp_train(esp_handle *h, const esp_lp_train_opts *o, double *loss)
{
    if (!h || !o) return ESP_EINVAL;
    if (!h->lp_weights) { h->err = "no network weights (esp_lp_init_weights / esp_lp_set_weights)"; return ESP_ESTATE; }
    if (h->lp_n <= 0) { h->err = "empty training set (esp_lp_collect)"; return ESP_ESTATE; }
    if (o->steps < 0 || o->batch < 8 || o->batch > (1 << 20) || !(o->lr > 0.0)) {
        h->err = "bad training options";
        return ESP_EINVAL;
    }
    const int B = (int)round8(o->batch);
    int rc = lp_ensure_batch(h, B);
    if (rc) return rc;
    if ((rc = lp_ensure_loss(h, std::max(1, o->steps)))) return rc;
    if (h->lp_engine == 1) CK(cudaMemsetAsync(h->d_tc_err, 0, sizeof(int), h->st));
    for (int s = 0; s < o->steps; ++s) {
        CK(launch_lp_gather(h->d_lp_x, h->d_lp_t, h->lp_n, B, o->seed, (uint64_t)(h->lp_adam_t), h->d_lp_xb,
                            h->d_lp_tb, h->st));
        if ((rc = lp_pass(h, B, B, h->d_lp_loss + s))) return rc;
        ++h->lp_adam_t;
        CK(launch_adam(h->d_lp_p, h->d_lp_g, h->d_lp_m, h->d_lp_v, kPadParams, (float)o->lr, (float)o->beta1,
                       (float)o->beta2, (float)o->eps, h->lp_adam_t, h->st));
        CK(launch_lp_to_bf16(h->d_lp_p, h->d_lp_w1, h->d_lp_w2, h->d_lp_w3, h->st));
        h->launches += 3;
    }
    if (loss && o->steps > 0) {
        if ((rc = d2h(h, loss, h->d_lp_loss, sizeof(double) * o->steps))) return rc;
    } else {
        CK(cudaStreamSynchronize(h->st));
    }
    return lp_tc_status(h, "esp_lp_train");
}

int esp_lp_loss_grad(esp_handle *h, const float *features, const float *targets, int64_t n, double *loss,
                     float *grad)
{
    if (!h || !features || !targets || n <= 0 || n > (1 << 20)) return ESP_EINVAL;
    if (!h->lp_weights) { h->err = "no network weights (esp_lp_init_weights / esp_lp_set_weights)"; return ESP_ESTATE; }
    const int B = (int)round8(n);
    int rc = lp_ensure_batch(h, B);
    if (rc) return rc;
    if ((rc = lp_ensure_loss(h, 1))) return rc;
    if (h->lp_engine == 1) CK(cudaMemsetAsync(h->d_tc_err, 0, sizeof(int), h->st));
    std::vector<__nv_bfloat16> x;
    bf16_rows(features, n, x);
    x.resize((size_t)B * kMlpInPad, __float2bfloat16_rn(0.f));   // zero rows up to the multiple of 8
    std::vector<float> t((size_t)B * 4, 0.f);
    std::memcpy(t.data(), targets, sizeof(float) * 4 * n);
    if ((rc = h2d(h, h->d_lp_xb, x.data(), sizeof(__nv_bfloat16) * x.size()))) return rc;
    if ((rc = h2d(h, h->d_lp_tb, t.data(), sizeof(float) * t.size()))) return rc;
    if ((rc = lp_pass(h, B, (int)n, h->d_lp_loss))) return rc;
    std::vector<float> g(kPadParams);
    if ((rc = d2h(h, g.data(), h->d_lp_g, sizeof(float) * kPadParams))) return rc;
    if (grad) lp_padded_to_logical(g, grad);
    if (loss && (rc = d2h(h, loss, h->d_lp_loss, sizeof(double)))) return rc;
    return lp_tc_status(h, "esp_lp_loss_grad");
}

int esp_lp_forward(esp_handle *h, const float *features, int64_t n, float *out)
{
    if (!h || !features || !out || n < 0 || n > (1 << 24)) return ESP_EINVAL;
    if (!h->lp_weights) { h->err = "no network weights (esp_lp_init_weights / esp_lp_set_weights)"; return ESP_ESTATE; }
    if (n == 0) return ESP_OK;
    std::vector<__nv_bfloat16> x;
    bf16_rows(features, n, x);
    __nv_bfloat16 *dx = nullptr;
    float *dout = nullptr;
    CK(dalloc(&dx, x.size()));
    cudaError_t e = dalloc(&dout, (size_t)n * kMlpOut);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x.data(), sizeof(__nv_bfloat16) * x.size(), cudaMemcpyHostToDevice, h->st);
    LpWeights w;
    w.w1 = h->d_lp_w1; w.w2 = h->d_lp_w2; w.w3 = h->d_lp_w3;
    w.b1 = h->d_lp_p + kPadB1; w.b2 = h->d_lp_p + kPadB2; w.b3 = h->d_lp_p + kPadB3;
    if (h->lp_engine == 1) {
        if (e == cudaSuccess) e = cudaMemsetAsync(h->d_tc_err, 0, sizeof(int), h->st);
        if (e == cudaSuccess)
            e = launch_lp_forward_tc(w, dx, (int)n, dout, h->d_tc_err, h->num_sms, h->st, h->tc_force_timeout);
    } else if (e == cudaSuccess) {
        e = launch_lp_forward(w, dx, (int)n, dout, h->st);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, sizeof(float) * n * kMlpOut, cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    h->launches++;
    dfree(dx); dfree(dout);
    if (e != cudaSuccess) { h->err = std::string("esp_lp_forward: ") + cudaGetErrorString(e); return ESP_ECUDA; }
    if (h->lp_engine == 1) {
        int flag = 0;
        int rc = d2h(h, &flag, h->d_tc_err, sizeof(int));
        if (rc) return rc;
        if (flag) { h->err = "esp_lp_forward: a tensor-core completion wait gave up"; return ESP_ETIMEOUT; }
    }
    return ESP_OK;
}

int esp_lp_set_engine(esp_handle *h, int32_t engine)
{
    if (!h || engine < 0 || engine > 1) return ESP_EINVAL;
    int rc = fold(h);
    if (rc) return rc;
    if (engine == 1 && !h->d_tc_err) {
        CK(dalloc(&h->d_tc_err, 1));
        CK(cudaMemsetAsync(h->d_tc_err, 0, sizeof(int), h->st));
    }
    if (engine == 1 && !h->d_lp_gwork) CK(dalloc(&h->d_lp_gwork, kGemmTcWorkFloats));
    h->lp_engine = engine;
    return ESP_OK;
}

int esp_lp_force_tc_timeout(esp_handle *h, int32_t on)
{
    if (!h) return ESP_EINVAL;
    int rc = fold(h);
    if (rc) return rc;
    h->tc_force_timeout = on ? 1 : 0;
    return ESP_OK;
}

int esp_set_proposal(esp_handle *h, int32_t kind)
{
    if (!h || kind < 0 || kind > 1) return ESP_EINVAL;
    if (kind == 1 && !h->lp_weights) {
        h->err = "the learned proposal needs network weights (esp_lp_init_weights / esp_lp_set_weights)";
        return ESP_ESTATE;
    }
    int rc = fold(h);
    if (rc) return rc;
    h->proposal = kind;
    return ESP_OK;
}

int esp_get_proposal(const esp_handle *h, int32_t *kind)
{
    if (!h || !kind) return ESP_EINVAL;
    *kind = h->proposal;
    return ESP_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batches: independent handles advanced together by one CUDA graph per
// `units_per_graph` measurement units, and the autotuner that picks each
// handle's sweep kernel and the units per graph by timing them.
// ---------------------------------------------------------------------------
struct esp_batch {
    std::vector<esp_handle *> hs;
    std::vector<cudaStream_t> prev;   // the handles' streams before the batch
    cudaStream_t st = nullptr;
    cudaStream_t own = nullptr;       // created when the caller passes no stream
    std::string err;
    int units_per_graph = 1;
    cudaGraphExec_t exec = nullptr;
    int exec_units = 0;
    struct Delta {
        int64_t c[4];
        long long const_hits, launches;
        // which spin copies are current before a replay (the graph relies on
        // them) and after it
        bool arrays_before, slab_before, arrays_after, slab_after;
    };
    std::vector<Delta> deltas;
};

namespace {

void mirrors(const esp_handle *h, int64_t c[4])
{
    c[0] = h->next_sweep; c[1] = h->next_swap; c[2] = h->run.meas_done; c[3] = h->run.units_done;
}

void set_mirrors(esp_handle *h, const int64_t c[4])
{
    h->next_sweep = c[0]; h->next_swap = c[1]; h->run.meas_done = c[2]; h->run.units_done = c[3];
}

void batch_drop_graph(esp_batch *b)
{
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
    b->exec_units = 0;
}

int batch_fail(esp_batch *b, const char *what, const esp_handle *h)
{
    b->err = std::string(what) + (h ? ": " + h->err : std::string());
    return ESP_ECUDA;
}

// Record K units of every handle into one graph.  The host counters are put
// back afterwards; each replay advances them by the recorded deltas.
int batch_capture(esp_batch *b, int K)
{
    batch_drop_graph(b);
    const size_t n = b->hs.size();
    std::vector<std::array<int64_t, 4>> base(n);
    std::vector<long long> hits0(n), launches0(n);
    for (size_t i = 0; i < n; ++i) {
        esp_handle *h = b->hs[i];
        if (!h->run.active) { b->err = "esp_begin has not been called on every handle"; return ESP_ESTATE; }
        int rc = fold(h);
        if (rc) return batch_fail(b, "fold", h);
        if (!h->d_ctr) {
            if (dalloc(&h->d_ctr, 4) != cudaSuccess) { b->err = "device allocation failed"; return ESP_ENOMEM; }
            h->ctr_valid = false;
        }
        // the graph is recorded from a fixed state of the spin copies, made
        // here outside the graph and restored before every replay: a handle
        // on the staged cluster path starts from its slab (the recorded
        // launches work on it), any other handle from its arrays
        if (use_cluster(h) && cluster_staged(h)) {
            rc = slab_current(h);
            h->arrays_ok = false;   // not relied upon by the graph
        } else {
            rc = arrays_current(h);
            h->slab_ok = false;
        }
        if (rc) return batch_fail(b, "spin copies", h);
        mirrors(h, base[i].data());
        hits0[i] = h->run.const_hits;
        launches0[i] = h->launches;
    }
    std::vector<std::array<bool, 2>> copies0(n);
    for (size_t i = 0; i < n; ++i) copies0[i] = {b->hs[i]->arrays_ok, b->hs[i]->slab_ok};
    cudaError_t e = cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) { b->err = std::string("cudaStreamBeginCapture: ") + cudaGetErrorString(e); return ESP_ECUDA; }
    for (size_t i = 0; i < n; ++i) {
        b->hs[i]->capturing = true;
        for (int c = 0; c < 4; ++c) b->hs[i]->cap_base[c] = base[i][c];
    }
    int rc = ESP_OK;
    const esp_handle *bad = nullptr;
    for (int k = 0; k < K && rc == ESP_OK; ++k)
        for (size_t i = 0; i < n && rc == ESP_OK; ++i)
            if ((rc = esp_advance(b->hs[i], 1))) bad = b->hs[i];
    b->deltas.assign(n, esp_batch::Delta{});
    for (size_t i = 0; i < n; ++i) {
        esp_handle *h = b->hs[i];
        int64_t now[4];
        mirrors(h, now);
        unsigned long long d[4];
        for (int c = 0; c < 4; ++c) {
            b->deltas[i].c[c] = now[c] - base[i][c];
            d[c] = (unsigned long long)b->deltas[i].c[c];
        }
        if (rc == ESP_OK && launch_bump(h->d_ctr, d, b->st) != cudaSuccess) { rc = ESP_ECUDA; bad = h; }
        b->deltas[i].const_hits = h->run.const_hits - hits0[i];
        b->deltas[i].launches = h->launches - launches0[i] + 1;
        b->deltas[i].arrays_before = copies0[i][0]; b->deltas[i].slab_before = copies0[i][1];
        b->deltas[i].arrays_after = h->arrays_ok; b->deltas[i].slab_after = h->slab_ok;
        h->arrays_ok = copies0[i][0]; h->slab_ok = copies0[i][1];
        set_mirrors(h, base[i].data());
        h->run.const_hits = hits0[i];
        h->launches = launches0[i];
        h->capturing = false;
    }
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(b->st, &g);
    if (rc != ESP_OK || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        if (rc == ESP_OK) b->err = std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e);
        else batch_fail(b, "capture", bad);
        return rc == ESP_OK ? ESP_ECUDA : rc;
    }
    e = cudaGraphInstantiate(&b->exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { b->exec = nullptr; b->err = std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e); return ESP_ECUDA; }
    b->exec_units = K;
    return ESP_OK;
}

int batch_replay(esp_batch *b)
{
    // the copies of the spins the graph was recorded with (a host call
    // between replays may have brought the arrays back or written them)
    for (size_t i = 0; i < b->hs.size(); ++i) {
        esp_handle *h = b->hs[i];
        const esp_batch::Delta &d = b->deltas[i];
        int rc = ESP_OK;
        if (d.slab_before && !h->slab_ok) rc = slab_current(h);
        if (rc == ESP_OK && d.arrays_before && !h->arrays_ok) rc = arrays_current(h);
        if (rc) return batch_fail(b, "spin copies", h);
    }
    for (esp_handle *h : b->hs) {
        int64_t now[4];
        mirrors(h, now);
        bool same = h->ctr_valid;
        for (int c = 0; c < 4; ++c) same = same && h->ctr_shadow[c] == (unsigned long long)now[c];
        if (!same) {
            for (int c = 0; c < 4; ++c) h->ctr_shadow[c] = (unsigned long long)now[c];
            cudaError_t e = cudaMemcpyAsync(h->d_ctr, h->ctr_shadow, sizeof(h->ctr_shadow), cudaMemcpyHostToDevice, b->st);
            if (e != cudaSuccess) { b->err = std::string("counter upload: ") + cudaGetErrorString(e); return ESP_ECUDA; }
            h->ctr_valid = true;
        }
    }
    cudaError_t e = cudaGraphLaunch(b->exec, b->st);
    if (e != cudaSuccess) { b->err = std::string("cudaGraphLaunch: ") + cudaGetErrorString(e); return ESP_ECUDA; }
    for (size_t i = 0; i < b->hs.size(); ++i) {
        esp_handle *h = b->hs[i];
        int64_t now[4];
        mirrors(h, now);
        for (int c = 0; c < 4; ++c) {
            now[c] += b->deltas[i].c[c];
            h->ctr_shadow[c] += (unsigned long long)b->deltas[i].c[c];
        }
        set_mirrors(h, now);
        h->run.const_hits += b->deltas[i].const_hits;
        h->launches += b->deltas[i].launches;
        h->arrays_ok = b->deltas[i].arrays_after;
        h->slab_ok = b->deltas[i].slab_after;
    }
    return ESP_OK;
}

int batch_advance(esp_batch *b, int64_t n)
{
    while (n > 0) {
        if (n >= b->units_per_graph) {
            if (b->exec_units != b->units_per_graph) {
                int rc = batch_capture(b, b->units_per_graph);
                if (rc) return rc;
            }
            int rc = batch_replay(b);
            if (rc) return rc;
            n -= b->exec_units;
        } else {
            for (esp_handle *h : b->hs) {
                int rc = esp_advance(h, 1);
                if (rc) return batch_fail(b, "esp_advance", h);
            }
            --n;
        }
    }
    return ESP_OK;
}

// Device time of `units` units of the whole batch (after one untimed unit).
int batch_time(esp_batch *b, int64_t units, double *us)
{
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess) return ESP_ECUDA;
    if (cudaEventCreate(&e1) != cudaSuccess) { cudaEventDestroy(e0); return ESP_ECUDA; }
    int rc = batch_advance(b, std::min<int64_t>(units, b->units_per_graph));
    if (!rc && cudaEventRecord(e0, b->st) != cudaSuccess) rc = ESP_ECUDA;
    if (!rc) rc = batch_advance(b, units);
    if (!rc && cudaEventRecord(e1, b->st) != cudaSuccess) rc = ESP_ECUDA;
    float ms = 0.f;
    if (!rc && (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)) rc = ESP_ECUDA;
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    if (rc == ESP_ECUDA && b->err.empty()) b->err = "event timing failed";
    *us = 1e3 * (double)ms / (double)units;
    return rc;
}

}  // namespace

extern "C" {

int esp_batch_create(esp_handle *const *handles, int32_t n, void *stream, esp_batch **out)
{
    if (!handles || n <= 0 || !out) { set_global_error("esp_batch_create: bad arguments"); return ESP_EINVAL; }
    *out = nullptr;
    for (int i = 0; i < n; ++i)
        if (!handles[i]) { set_global_error("esp_batch_create: null handle"); return ESP_EINVAL; }
    esp_batch *b = new (std::nothrow) esp_batch();
    if (!b) { set_global_error("host allocation failed"); return ESP_ENOMEM; }
    b->hs.assign(handles, handles + n);
    b->st = (cudaStream_t)stream;
    if (!b->st) {
        // graphs cannot be captured on the legacy default stream
        cudaError_t e = cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking);
        if (e != cudaSuccess) { set_global_error("cudaStreamCreate: %s", cudaGetErrorString(e)); delete b; return ESP_ECUDA; }
        b->st = b->own;
    }
    for (esp_handle *h : b->hs) {
        b->prev.push_back(h->st);
        int rc = esp_set_stream(h, (void *)b->st);
        if (rc) {
            set_global_error("esp_set_stream: %s", h->err.c_str());
            for (size_t i = 0; i + 1 < b->prev.size(); ++i) esp_set_stream(b->hs[i], (void *)b->prev[i]);
            if (b->own) cudaStreamDestroy(b->own);
            delete b;
            return rc;
        }
    }
    *out = b;
    return ESP_OK;
}

int esp_batch_destroy(esp_batch *b)
{
    if (!b) return ESP_EINVAL;
    if (b->st) cudaStreamSynchronize(b->st);
    batch_drop_graph(b);
    for (size_t i = 0; i < b->hs.size(); ++i) esp_set_stream(b->hs[i], (void *)b->prev[i]);
    if (b->own) cudaStreamDestroy(b->own);
    delete b;
    return ESP_OK;
}

int esp_batch_last_error(const esp_batch *b, char *buf, size_t len)
{
    if (!b || !buf || len == 0) return ESP_EINVAL;
    std::snprintf(buf, len, "%s", b->err.c_str());
    return ESP_OK;
}

int esp_batch_set_units_per_graph(esp_batch *b, int32_t units)
{
    if (!b || units < 1 || units > 4096) return ESP_EINVAL;
    if (units != b->units_per_graph) batch_drop_graph(b);
    b->units_per_graph = units;
    return ESP_OK;
}

int esp_batch_advance(esp_batch *b, int64_t units)
{
    if (!b || units < 0) return ESP_EINVAL;
    b->err.clear();
    return batch_advance(b, units);
}

int esp_batch_tune(esp_batch *b, int32_t units, esp_batch_tuning *out)
{
    if (!b || units < 1) return ESP_EINVAL;
    b->err.clear();
    const size_t n = b->hs.size();
    // 1. per handle: one colour class per launch (ELL kernel) or every colour
    //    and sweep of a unit in one launch (cluster-resident kernel) with the
    //    model's three best cluster geometries (CTAs per cluster, threads per CTA)
    for (size_t i = 0; i < n; ++i) {
        esp_handle *h = b->hs[i];
        if (h->proposal != 0) continue;
        struct Cand { int kind, cs, nt, S; };
        std::vector<Cand> cands{{1, 0, 0, 0}};
        if (h->cluster_ok) {
            const std::vector<ClusterGeom> g = cluster_candidates(h);
            for (size_t k = 0; k < g.size() && k < 3; ++k) cands.push_back({2, g[k].cs, g[k].nt, g[k].S});
        }
        if (h->tile_ok) {
            // kinds 4 + variant: cs, nt carry the tile edge and the replicas per
            // CTA (5, 6: the pipelined variants)
            const std::vector<TileGeom> g = tile_candidates(h);
            for (size_t k = 0; k < g.size() && k < 3; ++k) cands.push_back({4 + g[k].variant, g[k].T, g[k].G});
        }
        double best = 1e300, best_cl = 1e300;
        Cand pick{1, 0, 0, 0};
        for (const Cand &c : cands) {
            int rc = ESP_OK;
            if (c.kind == 2 && (rc = cluster_geometry(h, c.cs, c.nt, c.S))) return batch_fail(b, "cluster geometry", h);
            if (c.kind >= 4 && (rc = tile_geometry(h, c.cs, c.nt, c.kind - 4))) return batch_fail(b, "tile geometry", h);
            if ((rc = esp_set_sweep_kernel(h, std::min(c.kind, 4)))) return batch_fail(b, "esp_set_sweep_kernel", h);
            esp_batch one;
            one.hs.assign(1, h);
            one.st = b->st;
            double us = 0.0;
            rc = batch_time(&one, units, &us);
            batch_drop_graph(&one);
            if (rc) { b->err = one.err; return rc; }
            if (out && out->ell_us && c.kind == 1) out->ell_us[i] = us;
            if (c.kind != 1) best_cl = std::min(best_cl, us);
            if (us < best) { best = us; pick = c; }
        }
        if (out && out->cluster_us) out->cluster_us[i] = cands.size() > 1 ? best_cl : -1.0;
        int rc = ESP_OK;
        if (pick.kind == 2 && (rc = cluster_geometry(h, pick.cs, pick.nt, pick.S))) return batch_fail(b, "cluster geometry", h);
        if (pick.kind >= 4 && (rc = tile_geometry(h, pick.cs, pick.nt, pick.kind - 4)))
            return batch_fail(b, "tile geometry", h);
        if ((rc = esp_set_sweep_kernel(h, std::min(pick.kind, 4)))) return batch_fail(b, "esp_set_sweep_kernel", h);
        if (out && out->kernel) out->kernel[i] = std::min(pick.kind, 4);
        if (out && out->cluster_size) out->cluster_size[i] = h->cluster_ok ? h->csize : 0;
        if (out && out->cluster_threads) out->cluster_threads[i] = h->cluster_ok ? h->cthreads : 0;
        if (out && out->cluster_sites) out->cluster_sites[i] = h->cluster_ok ? h->csites : 0;
    }
    // 2. units per graph replay
    const int cands[4] = {1, 2, 4, 8};
    double best = 1e300;
    int best_u = 1;
    for (int c = 0; c < 4; ++c) {
        esp_batch_set_units_per_graph(b, cands[c]);
        double us = 0.0;
        const int64_t t_units = std::max<int64_t>(units, 2 * cands[c]);
        int rc = batch_time(b, t_units - t_units % cands[c], &us);
        if (rc) return rc;
        if (out && out->graph_us) out->graph_us[c] = us;
        if (us < best) { best = us; best_u = cands[c]; }
    }
    esp_batch_set_units_per_graph(b, best_u);
    if (out) { out->units_per_graph = best_u; out->us_per_unit = best; }
    return ESP_OK;
}

}  // extern "C"
