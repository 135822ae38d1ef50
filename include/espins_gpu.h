/*
 * espins_gpu.h -- C ABI of the GB300 Monte Carlo library (libespins_gpu.so).
 *
 * The library replaces the Monte Carlo hot path of ESpinS, which the Fortran
 * program reaches by direct calls from mc_prog (src/mc_prog.F90:170-186:
 * `call mcarlo_main()` / `call pt_main()`), with all data held in module
 * globals.  A Fortran host keeps param_read and jij_get/bij_get/dij_get,
 * hands the resulting ELL tables to esp_upload_tables, and calls esp_run in
 * place of mcarlo_main/pt_main, binding these entry points through an
 * iso_c_binding interface block (bind(C) functions and derived types).
 *
 * Conventions
 *  - Every entry point returns an int status: ESP_OK (0) or an ESP_E* code;
 *    esp_last_error() returns the message.  The Fortran shim passes a nonzero
 *    status to io_error (src/io.F90:217-266), which is how the reference stops.
 *  - Arrays use the reference's Fortran layouts: spin_matrix(3,N[,R]),
 *    jij_nbors_matrix(N,maxnb) (column-major, 1-based neighbour indices),
 *    dij_matrix(3,N,maxnb).  Energies are in Kelvin, as after jij.F90:163.
 *  - The caller owns every host array; the library copies what it needs.
 *    Device memory belongs to the handle.  One handle per host thread; calls
 *    on one handle are not thread-safe.  All work runs on the handle's CUDA
 *    stream (its own, or one given with esp_set_stream).
 *  - Device-side waits are bounded; a wait that runs out returns ESP_ETIMEOUT.
 */
#ifndef ESPINS_GPU_H
#define ESPINS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    ESP_OK = 0,
    ESP_EINVAL = 1,    /* bad argument or inconsistent tables */
    ESP_ECUDA = 2,     /* CUDA runtime error */
    ESP_ENOMEM = 3,    /* device allocation failed */
    ESP_ESTATE = 4,    /* call out of order (e.g. run before tables) */
    ESP_ETIMEOUT = 5,  /* a bounded device wait gave up */
    ESP_ECOLOR = 6     /* no valid colouring of the interaction graph */
};

typedef struct esp_handle esp_handle;

/* Sizes of one lattice (mc_parameters: num_total_atoms, num_atoms,
 * supercell_size, tems_num, boundary; src/parameters.F90:37-170). */
typedef struct {
    int32_t num_sites;      /* num_total_atoms = prod(supercell) * num_atoms */
    int32_t num_atoms;      /* atoms per unit cell */
    int32_t supercell[3];   /* supercell_size */
    int32_t num_replicas;   /* tems_num: one replica per temperature */
    int32_t open_boundary;  /* boundary = open (1) or periodic (0) */
} esp_dims;

/* The Hamiltonian as the reference's table builders leave it
 * (mc_jij jij.F90:32-39, mc_bij bij.F90:32-34, mc_dij dij.F90:32-34,
 * single-ion/field parameters.F90:129-131,926-995).  Absent terms: NULL. */
typedef struct {
    const double *mag;          /* mag_moments_matrix(N) */
    int32_t j_maxnb;            /* second extent of jij_matrix */
    const int32_t *j_nn;        /* jij_num_nbors_matrix(N) */
    const int32_t *j_nbors;     /* jij_nbors_matrix(N,maxnb), 1-based */
    const double *j_val;        /* jij_matrix(N,maxnb), Kelvin */
    int32_t b_maxnb;
    const int32_t *b_nn;        /* bij_num_nbors_matrix(N) or NULL */
    const int32_t *b_nbors;     /* bij_nbors_matrix(N,maxnb) */
    const double *b_val;        /* bij_matrix(N,maxnb) */
    int32_t d_maxnb;
    const int32_t *d_nn;        /* dij_num_nbors_matrix(N) or NULL */
    const int32_t *d_nbors;     /* dij_nbors_matrix(N,maxnb) */
    const double *d_val;        /* dij_matrix(3,N,maxnb) */
    const double *si_axis;      /* singleion_axes_cart(3,num_atoms) or NULL */
    const double *si_delta;     /* singleion_parameters(num_atoms), Kelvin */
    const double *field_axis;   /* field_axes_cart(3,num_atoms) or NULL */
    const double *field_val;    /* field_parameters(num_atoms), Kelvin */
} esp_tables;

/* The schedule of mcarlo (mcarlo.F90:496-659) or pt_mcarlo (pt.F90:524-942). */
typedef struct {
    int64_t steps_warmup;
    int64_t steps_mc;
    int64_t steps_measure;
    int32_t pt;                 /* 0: independent temperatures, 1: parallel tempering */
    int32_t mcarlo_mode;        /* 0: 'random' (uniform sphere), 1: 'const' (cone) */
    int64_t pt_steps_swap;
    double tilt_angles_max;
    uint64_t seed;              /* key of the Philox stream (replaces mtprng) */
    int32_t lbinerror;          /* binning_error */
    int32_t num_binning_level;
    const int32_t *binning_level;
} esp_schedule;

/* Results, caller-allocated.  R = num_replicas (temperatures), nf = num_freq
 * (esp_num_freq), nl = num_binning_level.  NULL members are skipped.
 * Values are normalised exactly as mcarlo.F90:713-733 / pt.F90:995-1024
 * normalise them before writing _mc.dat, _pm.dat and _binerror.dat. */
typedef struct {
    int64_t *rejected;          /* [R][2]: warm-up and measurement phase (pt: [R][2] = warmup2, main) */
    int64_t *steps_tot;         /* [2]: updates per temperature in each phase */
    double *energy;             /* [R][3]: initial, final by differences, final direct */
    double *data;               /* [R][6]: <E>,<E^2>,<E^4>,<|m|>,<m^2>,<m^4> */
    double *pm;                 /* [R][nf]: P(M) */
    double *binning;            /* [R][nl][2]: binning variances of E/N and |m| */
    int64_t *num_swaps;         /* [R][2]: tries, accepts (pt) */
    int32_t *map;               /* [R]: configuration index at each temperature, 1-based (pt) */
    int64_t steps_mc_eff;       /* steps_mc after pt rounding (pt.F90:537-544) */
} esp_results;

/* Options of one low-level sweep call. */
typedef struct {
    int32_t mcarlo_mode;        /* 0 random, 1 const */
    double tilt_angles_max;
    uint64_t seed;
    int32_t phase;              /* rejected-counter column: 0 or 1 */
} esp_sweep_opts;

/* ---- lifetime --------------------------------------------------------- */
/* Replaces the allocations of mcarlo_setup (mcarlo.F90:242-460) and
 * pt_setup (pt.F90:270-500). */
int esp_create(const esp_dims *dims, esp_handle **out);
int esp_destroy(esp_handle *h);
/* Message of the last failed call on h (or of esp_create when h is NULL). */
int esp_last_error(const esp_handle *h, char *buf, size_t len);
/* Launch on an existing CUDA stream (cudaStream_t) instead of the handle's
 * own; NULL selects the legacy default stream. */
int esp_set_stream(esp_handle *h, void *cuda_stream);

/* ---- data in ---------------------------------------------------------- */
/* Tables of jij_get/bij_get/dij_get (jij.F90:394-446 etc.) plus single-ion
 * and field data; builds the device ELL, merges duplicate neighbours, colours
 * the interaction graph and checks the colouring on the host. */
int esp_upload_tables(esp_handle *h, const esp_tables *t);
/* tems(R) in Kelvin, in the order of the temperature slots. */
int esp_set_temperatures(esp_handle *h, const double *tems);
/* spin_matrix(3,N,R) (mcarlo.F90:269-322, pt.F90:442-491).  The copy goes
 * through a staging area of pinned host and device memory (at most 256 MiB
 * each, two halves of whole temperature slots) that esp_upload_tables
 * allocates: the host copy of one block (on up to 16 threads) overlaps the
 * DMA and device-side conversion of the previous one.  Neither this call nor
 * esp_get_spins allocates. */
int esp_set_spins(esp_handle *h, const double *spins);
/* How esp_set_spins (bit 0) and esp_get_spins (bit 1) move the spins: a set
 * bit has one kernel read / write the caller's array directly, where the
 * device accesses pageable host memory through the host's page tables (a
 * coherent CPU-GPU link), a clear bit goes through the pinned staging; -1
 * restores the default (staged: on a GB300 the direct reads were barely
 * faster and direct writes into not yet touched pages fault each page in).
 * ESP_EINVAL for a direct mode on a device without that access.  No
 * counterpart in the reference. */
int esp_set_host_transfer(esp_handle *h, int32_t mode);
/* The mode in effect, and whether the device supports direct access. */
int esp_get_host_transfer(const esp_handle *h, int32_t *mode, int32_t *direct_supported);
/* Start configurations of the reference: 0 ferro (0,0,m), 1 rand
 * (theta = pi*u1, phi = 2 pi*u2, the same for every temperature as in
 * pt.F90:448-459), drawn from the Philox stream keyed by seed. */
int esp_init_spins(esp_handle *h, int32_t kind, uint64_t seed);

/* ---- the hot path ------------------------------------------------------ */
/* mcarlo_main / pt_main without file output: runs the whole schedule on the
 * device and fills *res. */
int esp_run(esp_handle *h, const esp_schedule *s, esp_results *res);
/* The same schedule in three parts, so a host can interleave its own work
 * (progress lines, energy series) with the measurement phase:
 *  esp_begin   zeroes the accumulators and runs the warm-up: plain sweeps
 *              (mcarlo.F90:506-521), or warm-up 1 and warm-up 2 with swaps
 *              (pt.F90:524-735);
 *  esp_advance runs n units of the measurement phase: a unit is one
 *              measurement (steps_measure sweeps + accumulators,
 *              mcarlo.F90:526-590) or, with pt, one swap interval
 *              (pt_steps_swap measurements followed by pt_swap, pt.F90:773-907);
 *  esp_collect computes the final direct energy and fills *res, normalised
 *              by the number of measurements made so far.
 * esp_run == esp_begin + esp_advance(all units of the schedule) + esp_collect. */
int esp_begin(esp_handle *h, const esp_schedule *s);
int esp_advance(esp_handle *h, int64_t n);
int esp_collect(esp_handle *h, esp_results *res);
/* n full sweeps (every colour once) of every replica, starting at global
 * sweep index first_sweep; the metropolis + delta_energy_get loop of
 * mcarlo.F90:511-535 in colour order. */
int esp_sweep(esp_handle *h, int64_t n, int64_t first_sweep, const esp_sweep_opts *o);
/* One colour class of one sweep (for parity checks of a single pass). */
int esp_sweep_colour(esp_handle *h, int32_t colour, int64_t sweep, const esp_sweep_opts *o);
/* pt_swap (pt.F90:1235-1288) on device: start = 1 or 2 (1-based first pair),
 * swap_index selects the Philox counter of the draws. */
int esp_pt_swap(esp_handle *h, int32_t start, int64_t swap_index, uint64_t seed);

/* ---- observables ------------------------------------------------------- */
/* energy_get (get_quant.F90:186-261) per temperature slot, FP64 accumulated;
 * also resets the running energies used by the sweeps to these values. */
int esp_energy(esp_handle *h, double *energy_out);
/* Running ("by adding differences") energies per temperature slot. */
int esp_running_energy(esp_handle *h, double *energy_out);
/* Running magnetisation sum_i s_i per temperature slot, [R][3]. */
int esp_running_magnetization(esp_handle *h, double *m_out);
/* ---- optional measurements ------------------------------------------- */
/* The order parameter and the staggered magnetisation of mcarlo.F90:553-578 /
 * pt.F90:808-838 (orderparam_get, staggered_get and the pdf_order /
 * pdf_staggered parts of Pm_get, get_quant.F90:366-493), measured with every
 * measurement of esp_advance / esp_run when chosen here:
 *   OP = sum_i s_i . a_type(i) / N   (a: orderparam_axes_cart, unit vectors)
 *   SM = |sum_i c_type(i) s_i| / N   (c: staggered_coeff, +1 or -1)
 * Call after esp_upload_tables (new tables clear the choice) and before
 * esp_begin; flags 0 switches both off.  orderparam_axes: [num_atoms][3]
 * (NULL unless ESP_OBS_ORDER_PARAMETER), staggered_coeff: [num_atoms] (NULL
 * unless ESP_OBS_STAGGERED). */
#define ESP_OBS_ORDER_PARAMETER 1
#define ESP_OBS_STAGGERED 2
int esp_set_observables(esp_handle *h, int32_t flags, const double *orderparam_axes,
                        const int32_t *staggered_coeff);

/* Caller-allocated; NULL members are skipped.  Normalised as the reference
 * normalises local_data columns 7-12, local_pm rows 2-3 and local_binning rows
 * 3-4 before writing _op.dat, _staggered.dat, _pm.dat and _binerror.dat
 * (mcarlo.F90:713-781, pt.F90:995-1048). */
typedef struct {
    double *data;               /* [R][6]: <|OP|>,<OP^2>,<OP^4>,<SM>,<SM^2>,<SM^4> */
    double *pm_op;              /* [R][nf]: P(OP) */
    double *pm_sm;              /* [R][nf]: P(SM) */
    double *binning;            /* [R][nl][2]: binning variances of |OP| and SM */
} esp_obs_results;
int esp_collect_observables(esp_handle *h, esp_obs_results *res);

/* Spin correlations of spincorr_get (get_quant.F90:495-540), measured with
 * every measurement when shells are set: per shell s and species pair (a, b)
 *   S   = sum_i sum_{j in shell s of i} s_i.s_j / (n_s(a, b) m_i m_j)
 *   A   = the same sum of |s_i.s_j| / (...)
 * with a = kind(i), b = kind(j), n_s(a, b) = shell_num_nbors_kind(s, a, b);
 * S, A and |S| are summed over measurements.  The tables are the reference's
 * Fortran arrays (column-major, 1-based indices):
 *   kind_atoms(N), shell_num_nbors_matrix(num_shells, N),
 *   shell_nbors_matrix(num_shells, N, nbors_max),
 *   shell_num_nbors_kind(num_shells, num_species, num_species)
 * (jij.F90:449-503).  At most 4096 bins (num_shells x num_species^2).  Call
 * after esp_upload_tables (new tables clear them) and before esp_begin;
 * num_shells 0 switches them off. */
int esp_set_spin_correlation(esp_handle *h, int32_t num_shells, int32_t num_species, int32_t nbors_max,
                             const int32_t *kind_atoms, const int32_t *shell_num_nbors,
                             const int32_t *shell_nbors, const int32_t *shell_num_nbors_kind);
/* [R][num_shells][num_species][num_species] each (C order: species of the
 * neighbour fastest), normalised as _spincorr.dat prints them: sums / (number
 * of measurements x N).  NULL outputs are skipped. */
int esp_collect_spin_correlation(esp_handle *h, double *spincorr, double *spincorr_abs, double *spincorr_tot_abs);

/* Structure factor of mcarlo_structure_factor (get_quant.F90:649-717),
 * measured after every measurement whose 1-based index is a multiple of
 * steps_measure (sfactor_steps_measure): per q-point the transverse
 * F(q) = sum_i (s_i - (s_i.q) q / q.q) e^{i q.r_i}, NSF = Re(p.F(q)) / |p|,
 * accumulating |F|^2, |F|^2 - NSF^2 and NSF^2.  qpts: [nq][3] cartesian
 * q-points (1/length, 2 pi included, the loop_xy order of the reference);
 * polar: sfactor_polar (cartesian); real_lattice(3,3) and
 * atoms_supercell_pos_cart(3,N) as the reference holds them (Fortran order,
 * a_j = real_lattice(j,:)).  The phase q.r is evaluated as whole lattice
 * translations in 32-bit fixed point plus an FP32 remainder, the sums in FP32.
 * Call after esp_upload_tables (new tables clear it) and before esp_begin;
 * nq 0 switches it off. */
int esp_set_structure_factor(esp_handle *h, int32_t nq, const double *qpts, const double *polar,
                             int32_t steps_measure, const double *real_lattice, const double *pos);
/* sf: [R][nq][3] divided by N and by the number of structure-factor
 * measurements (mcarlo.F90:821-822), which goes to *num_measured. */
int esp_collect_structure_factor(esp_handle *h, double *sf, int64_t *num_measured);

/* Local terms of every site: energy of site i as a function of its spin s is
 * g_i.s + s^T Q_i s;  g: (3,N,R), q: (6,N,R) as xx,yy,zz,xy,xz,yz.
 * The exchange local field of delta_energy_get is -g without the Zeeman part. */
int esp_local_terms(esp_handle *h, double *g_out, double *q_out);
int esp_get_spins(esp_handle *h, double *spins_out);
/* Colour of every site (0-based, N entries) and the number of colours. */
int esp_get_colouring(esp_handle *h, int32_t *colour_out, int32_t *num_colours);
/* Rejected counters per temperature slot, [R][2]. */
int esp_get_rejected(esp_handle *h, int64_t *rejected_out);
/* Temperature slot -> replica (0-based) after PT swaps. */
int esp_get_replica_of_slot(esp_handle *h, int32_t *replica_out);
/* Sweep kernel: 0 automatic, 1 the ELL kernel (any lattice), 2 the
 * cluster-resident kernel (periodic, translation-invariant lattices whose
 * replica fits the shared memory of one thread-block cluster), 4 the tiled
 * kernel (periodic, translation-invariant lattices with nearest-cell
 * couplings: cubes of T cells plus a one-cell halo of G replicas in shared
 * memory, updated in a 2x2x2 checkerboard of tiles).  ELL and cluster follow
 * the same colouring, random stream and summation order; the tiled kernel
 * uses the same random stream and arithmetic in tile order. */
int esp_set_sweep_kernel(esp_handle *h, int32_t kind);
/* Geometry of the cluster-resident sweep: CTAs per replica (slabs of z
 * planes), threads per CTA and sites of a colour pass each thread updates
 * together: (256, 1), (512, 1) or (512, 2); ESP_EINVAL where the lattice or
 * the GPU cannot run it.  Trajectories do not depend on it.  The getter
 * accepts sites_per_thread == NULL. */
int esp_set_cluster_geometry(esp_handle *h, int32_t cluster_size, int32_t threads, int32_t sites_per_thread);
int esp_get_cluster_geometry(const esp_handle *h, int32_t *cluster_size, int32_t *threads,
                             int32_t *sites_per_thread);
/* Geometry of the tiled sweep: tile edge in cells (even, 2 * tile dividing
 * every supercell edge), replicas per CTA, and the variant: 0 one CTA per
 * tile; persistent CTAs (tile 4, 6 or 8; 4, 8 or 16 replicas) that copy their
 * tiles asynchronously, 1 one per SM copying the next tile while updating the
 * current one, 2 two per SM (four of 128 threads for 4 replicas; at most 128
 * registers a thread) each copying, then updating, while the others update.
 * All give the same trajectory. */
int esp_set_tile_geometry(esp_handle *h, int32_t tile, int32_t replicas, int32_t pipelined);
int esp_get_tile_geometry(const esp_handle *h, int32_t *tile, int32_t *replicas, int32_t *pipelined);
/* The kernel in use (1 ELL, 2 cluster, 3 the learned-proposal sweep, 4
 * tiled) and the cluster size of the cluster path. */
int esp_get_sweep_kernel(const esp_handle *h, int32_t *kind, int32_t *cluster_size);
/* Keep the per-measurement series (E, |m|) of every temperature slot for
 * the last `capacity` measurements of a run (0 switches it off): the data of
 * the reference's energy series files (energy_write, get_quant.F90:1130-1223)
 * and of autocorrelation analyses. */
int esp_set_series(esp_handle *h, int64_t capacity);
/* *count = kept measurements; out (if not NULL) receives them oldest first,
 * out[(k*R + t)*2 + 0] = E, [.. + 1] = |m| of measurement k at slot t. */
int esp_get_series(esp_handle *h, double *out, int64_t *count);
/* num_freq of the P(M) grid (mcarlo.F90:432-442). */
int esp_num_freq(const esp_handle *h, int32_t *nf);
/* Number of kernels this handle has launched so far. */
int esp_launch_count(const esp_handle *h, int64_t *count);

/* ---- many independent lattices -------------------------------------------
 * No counterpart in the reference, which runs one lattice per invocation.
 * Lattices of the same shape and Hamiltonian share their tables: put them in
 * one handle as groups of replicas, each group its own temperature set, and
 * restrict replica exchange to the group (pt.F90:1235-1288 within each
 * lattice).  Lattices of different shapes live in different handles, which a
 * batch advances together. */
int esp_set_pt_groups(esp_handle *h, int32_t group_size);

/* A batch advances every handle (each after its own esp_begin) by whole
 * measurement units, recording `units_per_graph` units of all handles as one
 * CUDA graph and replaying it; kernels read their sweep, swap and
 * measurement indices from per-handle device counters that each replay
 * advances, so the random stream and the results are those of calling
 * esp_advance on every handle.  Every handle runs on `stream` (a
 * cudaStream_t; NULL: a stream the batch creates, since graphs cannot be
 * captured on the legacy default stream) until esp_batch_destroy gives the
 * handles their previous streams back. */
typedef struct esp_batch esp_batch;
typedef struct {
    int32_t units_per_graph;      /* chosen */
    double us_per_unit;           /* device time of one unit of the batch, chosen setting */
    int32_t *kernel;              /* [n] chosen sweep kernel per handle (1 ELL, 2 cluster, 4 tiled), or NULL */
    double *ell_us, *cluster_us;  /* [n] time per unit of each handle alone: ELL, and the best of the
                                     cluster / tiled candidates (-1: none possible), or NULL */
    double *graph_us;             /* [4] time per unit with 1, 2, 4, 8 units per graph, or NULL */
    int32_t *cluster_size, *cluster_threads;  /* [n] chosen cluster geometry per handle (0: none), or NULL */
    int32_t *cluster_sites;       /* [n] sites per thread of the chosen cluster geometry, or NULL */
} esp_batch_tuning;
int esp_batch_create(esp_handle *const *handles, int32_t n, void *stream, esp_batch **out);
int esp_batch_destroy(esp_batch *b);
int esp_batch_last_error(const esp_batch *b, char *buf, size_t len);
int esp_batch_set_units_per_graph(esp_batch *b, int32_t units);
int esp_batch_advance(esp_batch *b, int64_t units);
/* Autotuner: times every handle alone with each sweep kernel it supports
 * (one colour class per launch, or every colour and sweep of a unit per
 * launch with up to three cluster geometries) and keeps the fastest, then
 * times the whole batch with 1, 2, 4 and 8 units per graph and keeps the
 * fastest.  It advances every handle by about 25 * units measurement units,
 * which count as measurements of the run. */
int esp_batch_tune(esp_batch *b, int32_t units, esp_batch_tuning *out);

/* ---- learned proposal ------------------------------------------------------
 * No counterpart in the reference (whose trial spins are uniform on the sphere
 * or in a cone, get_quant.F90:80-162).  The trial spin of a site is drawn from
 * a 4-component von Mises-Fisher mixture whose parameters an MLP
 * (12 -> 128 -> 128 -> 20, ReLU, BF16 weights, FP32 accumulation) computes
 * from the site's environment (local field, quadratic form, beta) in a local
 * frame; the Metropolis-Hastings test uses the exact mixture density of the
 * old and the new spin, so the chain samples the same Boltzmann distribution.
 * The network is trained on the GPU on (environment, spin) pairs taken from
 * the plain sampler's configurations, by maximum likelihood (Adam).
 * Parameters travel as ESP_LP_NUM_PARAMS floats in the order
 * W1[128][12] b1[128] W2[128][128] b2[128] W3[20][128] b3[20] (row = output). */
#define ESP_LP_NUM_PARAMS 20756
typedef struct {
    int32_t steps;              /* optimiser steps */
    int32_t batch;              /* samples per step (rounded up to a multiple of 8) */
    double lr, beta1, beta2, eps;   /* Adam */
    uint64_t seed;              /* mini-batch draws */
} esp_lp_train_opts;
int esp_lp_num_params(void);
int esp_lp_init_weights(esp_handle *h, uint64_t seed);
int esp_lp_set_weights(esp_handle *h, const float *params);
int esp_lp_get_weights(esp_handle *h, float *params);
/* Training-set storage for `capacity` pairs (clears the set). */
int esp_lp_reserve(esp_handle *h, int64_t capacity);
/* Append the pairs of every site of one colour class in every replica of the
 * current configurations (until the storage is full); *rows = set size. */
int esp_lp_collect(esp_handle *h, int32_t colour, int64_t *rows);
/* Copy pairs [first, first+n) of the set: features (n,12) as stored (bf16
 * values), targets (n,4) = unit spin in the local frame and kappa0. */
int esp_lp_get_data(esp_handle *h, int64_t first, int64_t n, float *features, float *targets);
/* o->steps Adam steps on random mini-batches of the set; loss (if not NULL)
 * receives the mean negative log-likelihood of every step's batch. */
int esp_lp_train(esp_handle *h, const esp_lp_train_opts *o, double *loss);
/* Mean negative log-likelihood of n given pairs and its gradient with respect
 * to the parameters (ESP_LP_NUM_PARAMS floats), by the training kernels. */
int esp_lp_loss_grad(esp_handle *h, const float *features, const float *targets, int64_t n, double *loss,
                     float *grad);
/* Raw network outputs (n,20) of n feature rows by the sweep's fused forward pass. */
int esp_lp_forward(esp_handle *h, const float *features, int64_t n, float *out);
/* Tensor-core engine of the network in esp_lp_forward and the learned sweep:
 * 0 warp-level mma.sync tiles of 32 trials (default), 1 tcgen05 MMAs on
 * 128-trial tiles with tensor-memory accumulators.  ESP_ETIMEOUT if a
 * completion wait gave up. */
int esp_lp_set_engine(esp_handle *h, int32_t engine);
/* Test hook, no counterpart in the reference: with on != 0 every tcgen05
 * completion wait of the learned sweep and of esp_lp_forward reports that it
 * gave up, right after its first layer's MMAs have completed, so a host can
 * check the give-up path without a real hang: the sweep then makes no trial
 * and writes no spin, and esp_collect / esp_lp_forward return ESP_ETIMEOUT.
 * esp_begin clears the recorded give-up. */
int esp_lp_force_tc_timeout(esp_handle *h, int32_t on);
/* 0: the reference's trial moves (default); 1: the learned proposal (needs
 * weights).  Applies to esp_sweep, esp_sweep_colour, esp_run and esp_advance. */
int esp_set_proposal(esp_handle *h, int32_t kind);
int esp_get_proposal(const esp_handle *h, int32_t *kind);

/* ---- allocation-free direct energy ---------------------------------------
 * No counterpart in the reference: an extra entry point for hosts that own
 * all device memory and cannot let a library allocate (a Fortran program
 * whose arrays sit in its own device data regions, a framework with its own
 * caching allocator, a run that must not change its device footprint).
 * Every pointer below is a DEVICE pointer owned by the caller, in the
 * reference's layouts (as esp_tables, with spins = spin_matrix(3,N,R)).
 * The partial sums live in a 1 MiB array inside the library (held by every
 * GPU that loads it), so: num_replicas <= ESP_NOALLOC_MAX_REPLICAS and
 * num_sites * num_replicas < 2^31, else ESP_EINVAL.  The first call on each
 * device looks up that array's device address; make it before any stream
 * capture.  Calls that overlap on the GPU share the array and race. */
#define ESP_NOALLOC_MAX_REPLICAS 4096
typedef struct {
    int32_t num_sites, num_atoms, num_replicas;
    const double *spins;        /* (3,N,R) */
    const int32_t *j_nn, *j_nbors; const double *j_val;
    const int32_t *b_nn, *b_nbors; const double *b_val;   /* or NULL */
    const int32_t *d_nn, *d_nbors; const double *d_val;   /* or NULL */
    const double *si_axis, *si_delta;                     /* or NULL */
    const double *field_axis, *field_val;                 /* or NULL */
} esp_energy_args;
/* energy_out: device array [R]; runs on `stream` (a cudaStream_t, or NULL);
 * calls no cudaMalloc/cudaFree and allocates nothing. */
int esp_energy_noalloc(const esp_energy_args *a, double *energy_out, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* ESPINS_GPU_H */
