/*
 * espins_oracle.c -- FP64 CPU restatement of the ESpinS Monte Carlo hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA library in
 * espins_gb300/csrc: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline arm may load it.  Nothing in the product path links or calls it.
 *
 * It restates, in the reference's own FP64 arithmetic order, the routines of
 * ESpinS (Fortran 90) that form the Monte Carlo hot path:
 *
 *   MT19937 (mtprng)        src/mtprng.f90:152-173 (init), :227-282 (rand64),
 *                           :347-361 (real2)
 *   pair expansion to ELL   src/jij.F90:196-318,394-446; src/bij.F90:145-359;
 *                           src/dij.F90:145-391
 *   energy_get              src/get_quant.F90:186-261
 *   delta_energy_get        src/get_quant.F90:264-337
 *   metropolis              src/get_quant.F90:52-182
 *   magnetization_get       src/get_quant.F90:340-363
 *   Pm_get                  src/get_quant.F90:425-493
 *   orderparam_get          src/get_quant.F90:396-422
 *   staggered_get           src/get_quant.F90:366-392
 *   spincorr_get            src/get_quant.F90:495-540 (shells: jij.F90:449-503)
 *   mcarlo_structure_factor src/get_quant.F90:649-717
 *   mcarlo (one T chain)    src/mcarlo.F90:463-659 (+ grid :432-456)
 *   pt_mcarlo / pt_swap     src/pt.F90:504-942, :1235-1288
 *
 * It also holds a colour-ordered sweep driven by the same Philox4x32-10
 * counter stream the GPU kernels use (Salmon, Moraes, Dror, Shaw, "Parallel
 * random numbers: as easy as 1, 2, 3", SC'11), so a single GPU colour pass can
 * be compared update by update against an FP64 evaluation.
 *
 * Spins are stored as the reference stores spin_matrix(3,N): s[3*i+c].
 * ELL tables are 0-based and site-fastest: entry k of site i is at k*n+i,
 * which is the memory order of the Fortran arrays jij_nbors_matrix(N,maxnb).
 *
 * Build with -ffp-contract=off so the FP64 results do not depend on whether
 * the compiler fuses multiply-adds (aarch64 gcc fuses by default).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define OR_PI 3.141592653589793238462643383279
#define OR_TWOPI (2.0 * OR_PI)
#define OR_EPS4 1.0e-4
#define OR_EPS5 1.0e-5
#define OR_EPS8 1.0e-8

/* ------------------------------------------------------------------------ */
/* MT19937 exactly as mtprng.f90 generates it.                               */
/* ------------------------------------------------------------------------ */
typedef struct {
    int32_t mti;
    uint32_t mt[624];
} or_mt;

/* mtprng_init (mtprng.f90:152-173).  mt(0) holds the seed sign-extended to
 * 64 bits and mt(1) is formed from a LOGICAL 64-bit right shift by 30 of that
 * value, so for a negative seed the ones in bits 32..61 land in bits 2..31.
 * From mt(1) on every word is masked to 32 bits, and generation/tempering only
 * ever look at the low 32 bits, so storing the low words is exact. */
void or_mt_init(or_mt *st, int32_t seed)
{
    uint64_t m0 = (uint64_t)(int64_t)seed;
    st->mt[0] = (uint32_t)m0;
    uint64_t prev = m0;
    for (int i = 1; i < 624; ++i) {
        uint64_t v = (1812433253ULL * (prev ^ (prev >> 30)) + (uint64_t)i) & 0xffffffffULL;
        st->mt[i] = (uint32_t)v;
        prev = v;
    }
    st->mti = 624;
}

/* mtprng_rand64 (mtprng.f90:227-282): the standard MT19937 recurrence and
 * tempering on the low 32 bits. */
uint32_t or_mt_u32(or_mt *st)
{
    static const uint32_t mag01[2] = {0u, 0x9908b0dfu};
    uint32_t y;
    if (st->mti >= 624) {
        int kk;
        for (kk = 0; kk < 624 - 397; ++kk) {
            y = (st->mt[kk] & 0x80000000u) | (st->mt[kk + 1] & 0x7fffffffu);
            st->mt[kk] = st->mt[kk + 397] ^ (y >> 1) ^ mag01[y & 1u];
        }
        for (; kk < 623; ++kk) {
            y = (st->mt[kk] & 0x80000000u) | (st->mt[kk + 1] & 0x7fffffffu);
            st->mt[kk] = st->mt[kk + (397 - 624)] ^ (y >> 1) ^ mag01[y & 1u];
        }
        y = (st->mt[623] & 0x80000000u) | (st->mt[0] & 0x7fffffffu);
        st->mt[623] = st->mt[396] ^ (y >> 1) ^ mag01[y & 1u];
        st->mti = 0;
    }
    y = st->mt[st->mti++];
    y ^= (y >> 11);
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= (y >> 18);
    return y;
}

/* mtprng_rand_real2 (mtprng.f90:347-361): u32 / 2^32 in [0,1). */
double or_mt_real2(or_mt *st)
{
    return (double)or_mt_u32(st) * (1.0 / 4294967296.0);
}

/* ------------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon et al. SC'11), the GPU's counter-based stream.      */
/* ------------------------------------------------------------------------ */
void or_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4])
{
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* ------------------------------------------------------------------------ */
/* Hamiltonian tables                                                        */
/* ------------------------------------------------------------------------ */
typedef struct {
    int32_t n;          /* num_total_atoms */
    int32_t num_atoms;  /* atoms per unit cell */
    const double *mag;  /* mag_moments_matrix [n] */
    int32_t j_maxnb; const int32_t *j_nn; const int32_t *j_nb; const double *j_val;
    int32_t b_maxnb; const int32_t *b_nn; const int32_t *b_nb; const double *b_val;
    int32_t d_maxnb; const int32_t *d_nn; const int32_t *d_nb; const double *d_val; /* 3*(k*n+i)+c */
    int32_t have_si;    const double *si_axis; const double *si_delta; /* [3*num_atoms], [num_atoms] */
    int32_t have_field; const double *f_axis;  const double *f_val;
} or_ham;

static inline double dot3(const double *a, const double *b)
{
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

/* energy_get (get_quant.F90:186-261), same term order, then /2. */
double or_energy(const or_ham *h, const double *s)
{
    const int n = h->n;
    double e = 0.0;
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < h->j_nn[i]; ++k) {
            int j = h->j_nb[k * n + i];
            e = e - h->j_val[k * n + i] * dot3(s + 3 * i, s + 3 * j);
        }
    if (h->have_field)
        for (int i = 0; i < n; ++i) {
            int a = i % h->num_atoms;
            double sf = dot3(s + 3 * i, h->f_axis + 3 * a);
            e = e + 2.0 * h->f_val[a] * sf;
        }
    if (h->have_si)
        for (int i = 0; i < n; ++i) {
            int a = i % h->num_atoms;
            double sa = dot3(s + 3 * i, h->si_axis + 3 * a);
            e = e + 2.0 * h->si_delta[a] * sa * sa;
        }
    if (h->b_nn)
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < h->b_nn[i]; ++k) {
                int j = h->b_nb[k * n + i];
                double d = dot3(s + 3 * i, s + 3 * j);
                e = e + h->b_val[k * n + i] * d * d;
            }
    if (h->d_nn)
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < h->d_nn[i]; ++k) {
                int j = h->d_nb[k * n + i];
                const double *a = s + 3 * i, *b = s + 3 * j;
                double c[3];
                c[0] = a[1] * b[2] - a[2] * b[1];
                c[1] = a[2] * b[0] - a[0] * b[2];
                c[2] = a[0] * b[1] - a[1] * b[0];
                e = e + dot3(h->d_val + 3 * (k * n + i), c);
            }
    return e / 2.0;
}

/* delta_energy_get (get_quant.F90:264-337).  s already holds the NEW spin at
 * site i and ds = new - old; the old spin is re-formed as s_i - ds exactly as
 * the reference does. */
double or_delta_energy(const or_ham *h, int i, const double *s, const double *ds)
{
    const int n = h->n;
    double de = 0.0;
    for (int k = 0; k < h->j_nn[i]; ++k) {
        int j = h->j_nb[k * n + i];
        de = de - h->j_val[k * n + i] * dot3(ds, s + 3 * j);
    }
    if (h->have_field) {
        int a = i % h->num_atoms;
        de = de + h->f_val[a] * dot3(ds, h->f_axis + 3 * a);
    }
    if (h->have_si) {
        int a = i % h->num_atoms;
        double si[3] = {s[3 * i] - ds[0], s[3 * i + 1] - ds[1], s[3 * i + 2] - ds[2]};
        double sa = dot3(si, h->si_axis + 3 * a);
        double da = dot3(ds, h->si_axis + 3 * a);
        de = de + h->si_delta[a] * (da * da + 2.0 * sa * da);
    }
    if (h->b_nn)
        for (int k = 0; k < h->b_nn[i]; ++k) {
            int j = h->b_nb[k * n + i];
            double si[3] = {s[3 * i] - ds[0], s[3 * i + 1] - ds[1], s[3 * i + 2] - ds[2]};
            double sj = dot3(si, s + 3 * j);
            double dj = dot3(ds, s + 3 * j);
            de = de + h->b_val[k * n + i] * (dj * dj + 2.0 * sj * dj);
        }
    if (h->d_nn)
        for (int k = 0; k < h->d_nn[i]; ++k) {
            int j = h->d_nb[k * n + i];
            const double *b = s + 3 * j;
            double c[3];
            c[0] = ds[1] * b[2] - ds[2] * b[1];
            c[1] = ds[2] * b[0] - ds[0] * b[2];
            c[2] = ds[0] * b[1] - ds[1] * b[0];
            de = de + dot3(h->d_val + 3 * (k * n + i), c);
        }
    return de;
}

/* Local-field decomposition used by the GPU kernels: the energy of site i as
 * a function of its own spin s is  E_i(s) = g_i . s + s^T Q_i s  with
 *   g_i = -sum_k J_ik s_k + sum_k s_k x D_ik + f_i axis_i
 *   Q_i =  sum_k B_ik s_k s_k^T + Delta_i a_i a_i^T   (xx,yy,zz,xy,xz,yz)
 * Delta E of delta_energy_get equals E_i(new) - E_i(old) in exact arithmetic.
 * The exchange local field h_i = -g_i (without the Zeeman term) is what the
 * reference's exchange line computes against delta. */
void or_local_terms(const or_ham *h, const double *s, double *g, double *q)
{
    const int n = h->n;
    for (int i = 0; i < n; ++i) {
        double gx = 0, gy = 0, gz = 0;
        double qxx = 0, qyy = 0, qzz = 0, qxy = 0, qxz = 0, qyz = 0;
        for (int k = 0; k < h->j_nn[i]; ++k) {
            int j = h->j_nb[k * n + i];
            double J = h->j_val[k * n + i];
            gx -= J * s[3 * j]; gy -= J * s[3 * j + 1]; gz -= J * s[3 * j + 2];
        }
        if (h->d_nn)
            for (int k = 0; k < h->d_nn[i]; ++k) {
                int j = h->d_nb[k * n + i];
                const double *b = s + 3 * j, *D = h->d_val + 3 * (k * n + i);
                gx += b[1] * D[2] - b[2] * D[1];
                gy += b[2] * D[0] - b[0] * D[2];
                gz += b[0] * D[1] - b[1] * D[0];
            }
        if (h->have_field) {
            int a = i % h->num_atoms;
            gx += h->f_val[a] * h->f_axis[3 * a];
            gy += h->f_val[a] * h->f_axis[3 * a + 1];
            gz += h->f_val[a] * h->f_axis[3 * a + 2];
        }
        if (h->b_nn)
            for (int k = 0; k < h->b_nn[i]; ++k) {
                int j = h->b_nb[k * n + i];
                double B = h->b_val[k * n + i];
                const double *b = s + 3 * j;
                qxx += B * b[0] * b[0]; qyy += B * b[1] * b[1]; qzz += B * b[2] * b[2];
                qxy += B * b[0] * b[1]; qxz += B * b[0] * b[2]; qyz += B * b[1] * b[2];
            }
        if (h->have_si) {
            int a = i % h->num_atoms;
            const double *ax = h->si_axis + 3 * a;
            double D = h->si_delta[a];
            qxx += D * ax[0] * ax[0]; qyy += D * ax[1] * ax[1]; qzz += D * ax[2] * ax[2];
            qxy += D * ax[0] * ax[1]; qxz += D * ax[0] * ax[2]; qyz += D * ax[1] * ax[2];
        }
        g[3 * i] = gx; g[3 * i + 1] = gy; g[3 * i + 2] = gz;
        q[6 * i] = qxx; q[6 * i + 1] = qyy; q[6 * i + 2] = qzz;
        q[6 * i + 3] = qxy; q[6 * i + 4] = qxz; q[6 * i + 5] = qyz;
    }
}

/* metropolis (get_quant.F90:52-182).  mode 0 = 'random', 1 = 'const'. */
void or_metropolis(const or_ham *h, or_mt *st, int i, double beta, double *s,
                   double *energy, int64_t *rejected, int mode, double tilt)
{
    double mag = h->mag[i];
    double old[3] = {s[3 * i], s[3 * i + 1], s[3 * i + 2]};
    double ds[3];
    if (mode == 0) {
        double r = or_mt_real2(st);
        double cost = 2.0 * r - 1.0;
        double sint = sqrt(1.0 - cost * cost);
        r = or_mt_real2(st);
        double phi = r * OR_TWOPI;
        s[3 * i] = mag * sint * cos(phi);
        s[3 * i + 1] = mag * sint * sin(phi);
        s[3 * i + 2] = mag * cost;
    } else {
        double r = or_mt_real2(st);
        double theta = tilt * acos(2.0 * r - 1.0);
        r = or_mt_real2(st);
        double phi = r * OR_TWOPI;
        double sint = sin(theta);
        double sx = sint * cos(phi), sy = sint * sin(phi), sz = cos(theta);
        double sxy = sqrt(old[0] * old[0] + old[1] * old[1]);
        double cphi, sphi;
        if (sxy > OR_EPS8) { cphi = old[0] / sxy; sphi = old[1] / sxy; }
        else { cphi = 1.0; sphi = 0.0; }
        double nrm = sqrt(old[0] * old[0] + old[1] * old[1] + old[2] * old[2]);
        double on[3] = {1.0 / nrm * old[0], 1.0 / nrm * old[1], 1.0 / nrm * old[2]};
        s[3 * i] = mag * (cphi * on[2] * sx - sphi * sy + on[0] * sz);
        s[3 * i + 1] = mag * (sphi * on[2] * sx + cphi * sy + on[1] * sz);
        s[3 * i + 2] = mag * (-sqrt(on[0] * on[0] + on[1] * on[1]) * sx + on[2] * sz);
    }
    ds[0] = s[3 * i] - old[0]; ds[1] = s[3 * i + 1] - old[1]; ds[2] = s[3 * i + 2] - old[2];
    double de = or_delta_energy(h, i, s, ds);
    *energy = *energy + de;
    if (de > 0.0) {
        double fac = exp(-beta * de);
        double r = or_mt_real2(st);
        if (fac < r) {
            s[3 * i] = old[0]; s[3 * i + 1] = old[1]; s[3 * i + 2] = old[2];
            *energy = *energy - de;
            *rejected += 1;
        }
    }
}

/* magnetization_get (get_quant.F90:340-363): |sum_i s_i/N|^2. */
double or_magnetization2(const or_ham *h, const double *s)
{
    double m[3] = {0, 0, 0};
    double rn = (double)h->n;
    for (int j = 0; j < h->n; ++j) {
        m[0] = m[0] + s[3 * j] / rn;
        m[1] = m[1] + s[3 * j + 1] / rn;
        m[2] = m[2] + s[3 * j + 2] / rn;
    }
    return dot3(m, m);
}

/* num_freq of the P(M) grid (mcarlo.F90:432-442). */
int or_num_freq(const or_ham *h)
{
    double m_max = 0.0;
    for (int i = 0; i < h->num_atoms; ++i) m_max = m_max + fabs(h->mag[i]);
    double m_min = -m_max;
    int nf = (int)lround((m_max - m_min) / 0.01) + 1;
    if (nf == 1) nf = 2;
    return nf;
}

/* Pm_get (get_quant.F90:425-493), the P(M) part: per unit cell |sum s| binned
 * with nint onto num_freq points, each hit adding 1/d_m with d_m = 0.01.
 * Fortran's nint rounds half away from zero, which is C's lround. */
void or_pm(const or_ham *h, const double *s, int num_freq, double *pdf)
{
    double m_max = 0.0, d_m = 0.01;
    for (int i = 0; i < h->num_atoms; ++i) m_max = m_max + fabs(h->mag[i]);
    double m_min = -m_max;
    for (int j = 0; j < h->n; j += h->num_atoms) {
        double m[3] = {0, 0, 0};
        for (int i = 0; i < h->num_atoms; ++i) {
            m[0] = m[0] + s[3 * (j + i)];
            m[1] = m[1] + s[3 * (j + i) + 1];
            m[2] = m[2] + s[3 * (j + i) + 2];
        }
        double m2 = dot3(m, m);
        long p = lround(((sqrt(m2) - m_min) / (m_max - m_min)) * (double)(num_freq - 1)) + 1;
        if (p < 1) p = 1;
        pdf[p - 1] = pdf[p - 1] + 1.0 / d_m;
    }
}

/* orderparam_get (get_quant.F90:396-422): (sum_j s_j . a_type(j) / N)^2.
 * The reference's atom type of 1-based site j is mod(j, num_atoms) (0 read as
 * num_atoms), which is atom j % num_atoms of the cell for 0-based j. */
double or_orderparam2(const or_ham *h, const double *axes, const double *s)
{
    double op = 0.0, rn = (double)h->n;
    for (int j = 0; j < h->n; ++j)
        op = op + dot3(s + 3 * j, axes + 3 * (j % h->num_atoms)) / rn;
    return op * op;
}

/* staggered_get (get_quant.F90:366-392): |sum_j c_type(j) s_j / N|^2. */
double or_staggered2(const or_ham *h, const double *coeff, const double *s)
{
    double m[3] = {0, 0, 0}, rn = (double)h->n;
    for (int j = 0; j < h->n; ++j) {
        double c = coeff[j % h->num_atoms];
        for (int x = 0; x < 3; ++x) m[x] = m[x] + s[3 * j + x] * c / rn;
    }
    return dot3(m, m);
}

static inline void pm_hit(double v, double m_min, double m_max, int num_freq, double *pdf)
{
    long p = lround(((v - m_min) / (m_max - m_min)) * (double)(num_freq - 1)) + 1;
    if (p < 1) p = 1;
    if (p > num_freq) p = num_freq;   /* the reference does not guard the top */
    pdf[p - 1] = pdf[p - 1] + 1.0 / 0.01;
}

/* Pm_get (get_quant.F90:425-493), the pdf_order and pdf_staggered parts: per
 * unit cell the signed sum of s.a (order parameter) and |sum c s| (staggered
 * magnetisation), binned on the P(M) grid.  Either output may be NULL. */
void or_pm_obs(const or_ham *h, const double *s, int num_freq, const double *axes,
               const double *coeff, double *pdf_op, double *pdf_st)
{
    double m_max = 0.0;
    for (int i = 0; i < h->num_atoms; ++i) m_max = m_max + fabs(h->mag[i]);
    double m_min = -m_max;
    for (int j = 0; j < h->n; j += h->num_atoms) {
        if (pdf_op) {
            double op = 0.0;
            for (int i = 0; i < h->num_atoms; ++i) op = op + dot3(s + 3 * (j + i), axes + 3 * i);
            pm_hit(op, m_min, m_max, num_freq, pdf_op);
        }
        if (pdf_st) {
            double m[3] = {0, 0, 0};
            for (int i = 0; i < h->num_atoms; ++i)
                for (int x = 0; x < 3; ++x) m[x] = m[x] + s[3 * (j + i) + x] * coeff[i];
            pm_hit(sqrt(dot3(m, m)), m_min, m_max, num_freq, pdf_st);
        }
    }
}

/* Neighbour shells of spincorr_get (jij.F90:449-503), 0-based. */
typedef struct {
    int32_t num_shells, num_species, maxk;
    const int32_t *kind;    /* [n]: species of the site (kind_atoms - 1) */
    const int32_t *nn;      /* [S][n]: shell_num_nbors_matrix */
    const int32_t *nb;      /* [S][maxk][n]: shell_nbors_matrix, 0-based */
    const int32_t *count;   /* [S][nsp][nsp]: shell_num_nbors_kind(s, a, b) */
} or_shells;

/* spincorr_get (get_quant.F90:495-540): per shell and species pair (a, b)
 * of (site, neighbour) the sums of s_i.s_j and |s_i.s_j| over
 * shell_num_nbors_kind(s, a, b) m_i m_j; adds the signed sum to sc, its
 * magnitude to sc_tot and the sum of magnitudes to sc_abs ([S][nsp][nsp]). */
void or_spincorr(const or_ham *h, const or_shells *sh, const double *s, double *sc, double *sc_abs,
                 double *sc_tot)
{
    const int S = sh->num_shells, nsp = sh->num_species, n = h->n;
    double *tmp = (double *)calloc((size_t)2 * nsp * nsp, sizeof(double));
    double *tabs = tmp + (size_t)nsp * nsp;
    for (int is = 0; is < S; ++is) {
        memset(tmp, 0, sizeof(double) * 2 * (size_t)nsp * nsp);
        for (int i = 0; i < n; ++i) {
            int a = sh->kind[i];
            int cnt = sh->nn[(size_t)is * n + i];
            for (int k = 0; k < cnt; ++k) {
                int j = sh->nb[((size_t)is * sh->maxk + k) * n + i];
                int b = sh->kind[j];
                double d = dot3(s + 3 * i, s + 3 * j);
                double den = (double)sh->count[((size_t)is * nsp + a) * nsp + b] * h->mag[i] * h->mag[j];
                tmp[a * nsp + b] = tmp[a * nsp + b] + d / den;
                tabs[a * nsp + b] = tabs[a * nsp + b] + fabs(d) / den;
            }
        }
        for (int q = 0; q < nsp * nsp; ++q) {
            sc[(size_t)is * nsp * nsp + q] = sc[(size_t)is * nsp * nsp + q] + tmp[q];
            sc_tot[(size_t)is * nsp * nsp + q] = sc_tot[(size_t)is * nsp * nsp + q] + fabs(tmp[q]);
            sc_abs[(size_t)is * nsp * nsp + q] = sc_abs[(size_t)is * nsp * nsp + q] + tabs[q];
        }
    }
    free(tmp);
}

/* mcarlo_structure_factor (get_quant.F90:649-717) for one configuration:
 * for every q-point (cartesian, nq of them) the transverse sum
 * F(q) = sum_i (s_i - (s_i.q) q / q.q) exp(i q.r_i) and NSF, the REAL part of
 * sum_i p.(s_i - (s_i.q) q / q.q) exp(i q.r_i) / |p| (the reference stores it
 * in a real variable); adds |F|^2, |F|^2 - NSF^2 and NSF^2 to sf[3*iq + 0..2].
 * A q-point with all three components zero adds nothing. */
void or_structure_factor(const or_ham *h, const double *pos, int nq, const double *qpts, const double *polar,
                         const double *s, double *sf)
{
    const double pnorm = sqrt(dot3(polar, polar));
    for (int iq = 0; iq < nq; ++iq) {
        const double *q = qpts + 3 * iq;
        if (q[0] == 0.0 && q[1] == 0.0 && q[2] == 0.0) continue;
        const double qq = dot3(q, q);
        double fre[3] = {0, 0, 0}, fim[3] = {0, 0, 0};
        double nsf = 0.0;
        for (int i = 0; i < h->n; ++i) {
            const double qr = dot3(pos + 3 * i, q);
            const double c = cos(qr), sn = sin(qr);
            const double mq = dot3(s + 3 * i, q) / qq;
            double v[3];
            for (int x = 0; x < 3; ++x) {
                v[x] = s[3 * i + x] - mq * q[x];
                fre[x] = fre[x] + v[x] * c;
                fim[x] = fim[x] + v[x] * sn;
            }
            nsf = nsf + dot3(polar, v) * c / pnorm;
        }
        const double f2 = fre[0] * fre[0] + fim[0] * fim[0] + fre[1] * fre[1] + fim[1] * fim[1]
                        + fre[2] * fre[2] + fim[2] * fim[2];
        sf[3 * iq] = sf[3 * iq] + f2;
        sf[3 * iq + 1] = sf[3 * iq + 1] + f2 - nsf * nsf;
        sf[3 * iq + 2] = sf[3 * iq + 2] + nsf * nsf;
    }
}

/* The optional measurements of one temperature slot after a measurement
 * (mcarlo.F90:553-578, pt.F90:808-838): sums of |x|, x^2, x^4 with x^2 the
 * squared order parameter (data[0..2]) and staggered magnetisation
 * (data[3..5]); binning partial sums ls[nlev][2]; P(OP) and P(SM). */
typedef struct {
    const double *op_axes;  /* orderparam_axes_cart(3,num_atoms), unit vectors, or NULL */
    const double *st_coeff; /* staggered_coeff(num_atoms) (+1/-1), or NULL */
    double *data;           /* [R][6], caller-zeroed */
    double *pm_op, *pm_st;  /* [R][num_freq] or NULL, caller-zeroed */
    double *binning;        /* [R][nlev][2] or NULL, caller-zeroed: binning variances of |OP| and |SM| */
    const or_shells *shells;            /* spin correlations, or NULL */
    double *sc, *sc_abs, *sc_tot;       /* [R][S][nsp][nsp], caller-zeroed */
} or_obs;

static void obs_measure(const or_ham *h, const or_obs *ob, int t, const double *s, int nf,
                        int nlev, double *ls)
{
    double *d = ob->data + 6 * (size_t)t;
    if (ob->op_axes) {
        double o2 = or_orderparam2(h, ob->op_axes, s);
        d[0] = d[0] + sqrt(o2); d[1] = d[1] + o2; d[2] = d[2] + o2 * o2;
        if (ls) for (int l = 0; l < nlev; ++l) ls[2 * l] = ls[2 * l] + sqrt(o2);
    }
    if (ob->st_coeff) {
        double m2 = or_staggered2(h, ob->st_coeff, s);
        d[3] = d[3] + sqrt(m2); d[4] = d[4] + m2; d[5] = d[5] + m2 * m2;
        if (ls) for (int l = 0; l < nlev; ++l) ls[2 * l + 1] = ls[2 * l + 1] + sqrt(m2);
    }
    if (ob->shells) {
        size_t B = (size_t)ob->shells->num_shells * ob->shells->num_species * ob->shells->num_species;
        or_spincorr(h, ob->shells, s, ob->sc + B * t, ob->sc_abs + B * t, ob->sc_tot + B * t);
    }
    if ((ob->pm_op && ob->op_axes) || (ob->pm_st && ob->st_coeff))
        or_pm_obs(h, s, nf, ob->op_axes,  ob->st_coeff,
                  ob->pm_op && ob->op_axes ? ob->pm_op + (size_t)nf * t : NULL,
                  ob->pm_st && ob->st_coeff ? ob->pm_st + (size_t)nf * t : NULL);
}

/* A completed binning block of level l: divide, square into the variance sum. */
static void obs_block(const or_obs *ob, int t, int nlev, int l, double div, double *ls)
{
    double *bn = ob->binning + ((size_t)t * nlev + l) * 2;
    for (int c = 0; c < 2; ++c) {
        ls[2 * l + c] = ls[2 * l + c] / div;
        bn[c] = bn[c] + ls[2 * l + c] * ls[2 * l + c];
        ls[2 * l + c] = 0.0;
    }
}

/* mcarlo.F90:635-656 for the |OP| and |SM| rows (pt: pt.F90:914-936, with
 * the extra 1/N). */
static void obs_finish(const or_obs *ob, int t, int nlev, const int32_t *levels, int64_t steps_mc,
                       double *ls, int n_div)
{
    const double *d = ob->data + 6 * (size_t)t;
    for (int l = 0; l < nlev; ++l) {
        double *bn = ob->binning + ((size_t)t * nlev + l) * 2;
        ls[2 * l] = d[0] - ls[2 * l];
        ls[2 * l + 1] = d[3] - ls[2 * l + 1];
        int64_t blk = (int64_t)1 << levels[l];
        int64_t m_l = steps_mc / blk;
        for (int c = 0; c < 2; ++c) {
            double v = ls[2 * l + c] / (double)blk;
            v = v / (double)m_l;
            double b = bn[c] / (double)m_l;
            b = (b - v * v) / (double)(m_l - 1);
            if (n_div > 0) b = b / (double)n_div;
            bn[c] = b;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Plain Metropolis for one temperature (mcarlo.F90:496-659).                */
/* ------------------------------------------------------------------------ */
typedef struct {
    int64_t steps_warmup, steps_mc, steps_measure;
    int32_t mode;          /* 0 random, 1 const */
    double tilt;
    int32_t num_binning_level;
    const int32_t *binning_level;
} or_mc_opts;

typedef struct {
    int64_t rejected[2];    /* warmup, mc */
    int64_t steps_tot[2];
    double energy[3];       /* initial, final by differences, final direct */
    double data[6];         /* E, E2, E4, M, M2, M4 (sums, not normalised) */
    double *pm;             /* [num_freq] caller-allocated, accumulated */
    double *binning;        /* [2*nlev] caller-allocated: local_binning(1:2,l) */
    const or_obs *obs;      /* order parameter / staggered magnetisation, or NULL (R = 1) */
} or_mc_result;

void or_mcarlo_run(const or_ham *h, const or_mc_opts *o, or_mt *st, double beta,
                   double *s, or_mc_result *res)
{
    const int n = h->n;
    const int nlev = o->num_binning_level;
    int nf = or_num_freq(h);
    double *lsum = (double *)calloc((size_t)(2 * (nlev > 0 ? nlev : 1)), sizeof(double));
    double *lso = (double *)calloc((size_t)(2 * (nlev > 0 ? nlev : 1)), sizeof(double));
    const or_obs *ob = res->obs;
    memset(res->data, 0, sizeof(res->data));
    res->rejected[0] = res->rejected[1] = 0;
    res->steps_tot[0] = res->steps_tot[1] = 0;
    if (res->binning) memset(res->binning, 0, sizeof(double) * 2 * nlev);
    double e = or_energy(h, s);
    res->energy[0] = e;
    for (int64_t mc = 0; mc < o->steps_warmup; ++mc)
        for (int64_t ms = 0; ms < o->steps_measure; ++ms)
            for (int i = 0; i < n; ++i) {
                or_metropolis(h, st, i, beta, s, &e, &res->rejected[0], o->mode, o->tilt);
                res->steps_tot[0]++;
            }
    for (int64_t mc = 1; mc <= o->steps_mc; ++mc) {
        for (int64_t ms = 0; ms < o->steps_measure; ++ms)
            for (int i = 0; i < n; ++i) {
                or_metropolis(h, st, i, beta, s, &e, &res->rejected[1], o->mode, o->tilt);
                res->steps_tot[1]++;
            }
        double e2 = e * e;
        res->data[0] = res->data[0] + e;
        res->data[1] = res->data[1] + e2;
        res->data[2] = res->data[2] + e2 * e2;
        double m2 = or_magnetization2(h, s);
        res->data[3] = res->data[3] + sqrt(m2);
        res->data[4] = res->data[4] + m2;
        res->data[5] = res->data[5] + m2 * m2;
        if (res->binning) {
            for (int l = 0; l < nlev; ++l) {
                lsum[2 * l] = lsum[2 * l] + e / (double)n;
                lsum[2 * l + 1] = lsum[2 * l + 1] + sqrt(m2);
            }
        }
        if (ob) obs_measure(h, ob, 0, s, nf, nlev, res->binning && ob->binning ? lso : NULL);
        if (res->pm) or_pm(h, s, nf, res->pm);
        if (res->binning) {
            for (int l = 0; l < nlev; ++l) {
                int64_t blk = (int64_t)1 << o->binning_level[l];
                if (mc % blk == 0) {
                    for (int c = 0; c < 2; ++c) {
                        lsum[2 * l + c] = lsum[2 * l + c] / (double)blk;
                        res->binning[2 * l + c] = res->binning[2 * l + c] + lsum[2 * l + c] * lsum[2 * l + c];
                        lsum[2 * l + c] = 0.0;
                    }
                    if (ob && ob->binning) obs_block(ob, 0, nlev, l, (double)blk, lso);
                }
            }
        }
    }
    if (res->binning) {
        for (int l = 0; l < nlev; ++l) {
            lsum[2 * l] = res->data[0] / (double)n - lsum[2 * l];
            lsum[2 * l + 1] = res->data[3] - lsum[2 * l + 1];
            int64_t blk = (int64_t)1 << o->binning_level[l];
            int64_t m_l = o->steps_mc / blk;
            for (int c = 0; c < 2; ++c) {
                double v = lsum[2 * l + c] / (double)blk;
                v = v / (double)m_l;
                double b = res->binning[2 * l + c] / (double)m_l;
                res->binning[2 * l + c] = (b - v * v) / (double)(m_l - 1);
            }
        }
        if (ob && ob->binning) obs_finish(ob, 0, nlev, o->binning_level, o->steps_mc, lso, 0);
    }
    res->energy[1] = e;
    res->energy[2] = or_energy(h, s);
    free(lsum);
    free(lso);
}

/* ------------------------------------------------------------------------ */
/* Parallel tempering, single stream (pt.F90:504-942, pt_swap :1235-1288).   */
/* ------------------------------------------------------------------------ */
typedef struct {
    int64_t steps_warmup, steps_mc, steps_measure, pt_steps_swap;
    int32_t mode;
    double tilt;
    int32_t num_binning_level;
    const int32_t *binning_level;
} or_pt_opts;

typedef struct {
    int64_t *rejected;      /* [R] main-phase rejects per temperature slot */
    int64_t *num_swaps;     /* [2*R] tries, accepts (main phase) */
    int32_t *map;           /* [R] 1-based configuration map */
    double *energy;         /* [3*R] */
    double *data;           /* [6*R] sums */
    double *pm;             /* [R*num_freq] */
    double *binning;        /* [R*2*nlev] */
    const or_obs *obs;      /* order parameter / staggered magnetisation, or NULL */
    int64_t steps_mc_eff;   /* steps_mc after rounding to pt_steps_swap */
    int64_t steps_tot_main; /* per-slot updates in the main phase */
} or_pt_result;

void or_pt_swap(int start1, int R, const double *tems, int n, double *spins,
                double *energy2, int32_t *map, int64_t *num_swap, or_mt *st, double *tmp)
{
    for (int l = start1; l <= R - 1; l += 2) {
        int a = l - 1, b = l;
        int swap = 0;
        double fac = (1.0 / tems[a] - 1.0 / tems[b]) * (energy2[a] - energy2[b]);
        num_swap[2 * a] += 1;
        num_swap[2 * b] += 1;
        if (fac > 0.0) swap = 1;
        else {
            double r = or_mt_real2(st);
            if (r < exp(fac)) swap = 1;
        }
        if (swap) {
            memcpy(tmp, spins + (size_t)3 * n * a, sizeof(double) * 3 * n);
            memcpy(spins + (size_t)3 * n * a, spins + (size_t)3 * n * b, sizeof(double) * 3 * n);
            memcpy(spins + (size_t)3 * n * b, tmp, sizeof(double) * 3 * n);
            double t = energy2[a]; energy2[a] = energy2[b]; energy2[b] = t;
            int32_t im = map[a]; map[a] = map[b]; map[b] = im;
            num_swap[2 * a + 1] += 1;
            num_swap[2 * b + 1] += 1;
        }
    }
}

static int64_t ceil_div_real(int64_t a, int64_t b)
{
    /* ceiling(real(a)/real(b)) for a >= 0, b > 0 */
    return (a + b - 1) / b;
}

void or_pt_run(const or_ham *h, const or_pt_opts *o, or_mt *st, int R,
               const double *tems, double *spins, or_pt_result *res)
{
    const int n = h->n;
    const int nlev = o->num_binning_level;
    int nf = or_num_freq(h);
    double *tmp = (double *)malloc(sizeof(double) * 3 * (size_t)n);
    double *e2 = (double *)calloc((size_t)R, sizeof(double));
    double *lsum = (double *)calloc((size_t)R * 2 * (nlev > 0 ? nlev : 1), sizeof(double));
    double *lso = (double *)calloc((size_t)R * 2 * (nlev > 0 ? nlev : 1), sizeof(double));
    const or_obs *ob = res->obs;
    int64_t pss = o->pt_steps_swap;
    int64_t sw = ceil_div_real(o->steps_warmup, 2);
    int64_t nsw_warm = ceil_div_real(sw, pss);
    sw = nsw_warm * pss;
    int64_t nsw = ceil_div_real(o->steps_mc, pss);
    int64_t steps_mc = nsw * pss;
    res->steps_mc_eff = steps_mc;
    for (int t = 0; t < R; ++t) res->map[t] = t + 1;
    memset(res->num_swaps, 0, sizeof(int64_t) * 2 * R);
    memset(res->rejected, 0, sizeof(int64_t) * R);
    memset(res->data, 0, sizeof(double) * 6 * R);
    if (res->binning) memset(res->binning, 0, sizeof(double) * 2 * nlev * R);
    if (sw > 0) {
        for (int t = 0; t < R; ++t) {
            double beta = 1.0 / tems[t];
            double *s = spins + (size_t)3 * n * t;
            e2[t] = or_energy(h, s);
            for (int64_t mc = 0; mc < sw; ++mc)
                for (int64_t ms = 0; ms < o->steps_measure; ++ms)
                    for (int i = 0; i < n; ++i)
                        or_metropolis(h, st, i, beta, s, &e2[t], &res->rejected[t], o->mode, o->tilt);
        }
        memset(res->rejected, 0, sizeof(int64_t) * R);
        for (int64_t lsw = 1; lsw <= nsw_warm; ++lsw) {
            for (int t = 0; t < R; ++t) {
                double beta = 1.0 / tems[t];
                double *s = spins + (size_t)3 * n * t;
                for (int64_t mc = 0; mc < pss; ++mc)
                    for (int64_t ms = 0; ms < o->steps_measure; ++ms)
                        for (int i = 0; i < n; ++i)
                            or_metropolis(h, st, i, beta, s, &e2[t], &res->rejected[t], o->mode, o->tilt);
            }
            int start = (int)((lsw + 1) % 2) + 1;
            or_pt_swap(start, R, tems, n, spins, e2, res->map, res->num_swaps, st, tmp);
        }
    } else {
        for (int t = 0; t < R; ++t) e2[t] = or_energy(h, spins + (size_t)3 * n * t);
    }
    for (int t = 0; t < R; ++t) res->energy[3 * t] = e2[t];
    memset(res->rejected, 0, sizeof(int64_t) * R);
    memset(res->num_swaps, 0, sizeof(int64_t) * 2 * R);
    int64_t steps_tot = 0;
    for (int64_t lsw = 1; lsw <= nsw; ++lsw) {
        for (int t = 0; t < R; ++t) {
            double beta = 1.0 / tems[t];
            double *s = spins + (size_t)3 * n * t;
            steps_tot = 0;
            for (int64_t mc = 1; mc <= pss; ++mc) {
                int64_t num_steps = (lsw - 1) * pss + mc;
                for (int64_t ms = 0; ms < o->steps_measure; ++ms)
                    for (int i = 0; i < n; ++i) {
                        or_metropolis(h, st, i, beta, s, &e2[t], &res->rejected[t], o->mode, o->tilt);
                        steps_tot++;
                    }
                double e = e2[t], ee = e * e;
                double *d = res->data + 6 * t;
                d[0] = d[0] + e; d[1] = d[1] + ee; d[2] = d[2] + ee * ee;
                double m2 = or_magnetization2(h, s);
                d[3] = d[3] + sqrt(m2); d[4] = d[4] + m2; d[5] = d[5] + m2 * m2;
                if (ob) obs_measure(h, ob, t, s, nf, nlev, res->binning && ob->binning ? lso + (size_t)2 * nlev * t : NULL);
                if (res->binning) {
                    double *ls = lsum + (size_t)2 * nlev * t;
                    double *bn = res->binning + (size_t)2 * nlev * t;
                    for (int l = 0; l < nlev; ++l) {
                        ls[2 * l] = ls[2 * l] + e / (double)n;
                        ls[2 * l + 1] = ls[2 * l + 1] + sqrt(m2);
                    }
                    for (int l = 0; l < nlev; ++l) {
                        int64_t blk = (int64_t)1 << o->binning_level[l];
                        if (num_steps % blk == 0) {
                            /* pt.F90:844 divides by 2**l (the level's position) */
                            double div = (double)((int64_t)1 << (l + 1));
                            for (int c = 0; c < 2; ++c) {
                                ls[2 * l + c] = ls[2 * l + c] / div;
                                bn[2 * l + c] = bn[2 * l + c] + ls[2 * l + c] * ls[2 * l + c];
                                ls[2 * l + c] = 0.0;
                            }
                            if (ob && ob->binning) obs_block(ob, t, nlev, l, div, lso + (size_t)2 * nlev * t);
                        }
                    }
                }
                if (res->pm) or_pm(h, s, nf, res->pm + (size_t)nf * t);
            }
        }
        int start = (int)((lsw + 1) % 2) + 1;
        or_pt_swap(start, R, tems, n, spins, e2, res->map, res->num_swaps, st, tmp);
    }
    res->steps_tot_main = nsw * steps_tot;
    if (res->binning) {
        for (int t = 0; t < R; ++t) {
            double *ls = lsum + (size_t)2 * nlev * t;
            double *bn = res->binning + (size_t)2 * nlev * t;
            const double *d = res->data + 6 * t;
            for (int l = 0; l < nlev; ++l) {
                ls[2 * l] = d[0] / (double)n - ls[2 * l];
                ls[2 * l + 1] = d[3] - ls[2 * l + 1];
                int64_t blk = (int64_t)1 << o->binning_level[l];
                int64_t m_l = steps_mc / blk;
                for (int c = 0; c < 2; ++c) {
                    double v = ls[2 * l + c] / (double)blk;
                    v = v / (double)m_l;
                    double b = bn[2 * l + c] / (double)m_l;
                    b = (b - v * v) / (double)(m_l - 1);
                    bn[2 * l + c] = b / (double)n;
                }
            }
            if (ob && ob->binning) obs_finish(ob, t, nlev, o->binning_level, steps_mc, lso + (size_t)2 * nlev * t, n);
        }
    }
    for (int t = 0; t < R; ++t) {
        res->energy[3 * t + 1] = e2[t];
        res->energy[3 * t + 2] = or_energy(h, spins + (size_t)3 * n * t);
    }
    free(tmp); free(e2); free(lsum); free(lso);
}

/* ------------------------------------------------------------------------ */
/* Colour-ordered sweep on the GPU's Philox stream (FP64 arithmetic).        */
/*                                                                           */
/* Update of site i of replica r in sweep w draws                            */
/*   x = Philox4x32-10(ctr = {i, r, lo32(w), hi32(w)}, key = {seed_lo, seed_hi})*/
/* and uses u_k = (x_k >> 8) * 2^-24:                                        */
/*   random mode: cos(theta) = 2 u0 - 1, phi = 2 pi u1                        */
/*   const mode : theta = tilt * acos(2 u0 - 1), phi = 2 pi u1, rotated onto  */
/*                the old direction as get_quant.F90:94-162 does              */
/*   accept     : dE <= 0, or exp(-beta dE) >= u2                             */
/* Sites of one colour never share a bond, so their order inside a colour    */
/* does not matter.  accept_out (optional, [n]) receives 1/0 per site of the  */
/* colour, -1 for sites of other colours.                                     */
/* ------------------------------------------------------------------------ */
static inline double u24(uint32_t x) { return (double)(x >> 8) * (1.0 / 16777216.0); }

void or_trial_spin(const double *old, double mag, int mode, double tilt,
                   const uint32_t x[4], double *out)
{
    double u0 = u24(x[0]), u1 = u24(x[1]);
    if (mode == 0) {
        double c = 2.0 * u0 - 1.0;
        double sn = sqrt(fmax(0.0, 1.0 - c * c));
        double phi = OR_TWOPI * u1;
        out[0] = mag * sn * cos(phi);
        out[1] = mag * sn * sin(phi);
        out[2] = mag * c;
    } else {
        double theta = tilt * acos(2.0 * u0 - 1.0);
        double phi = OR_TWOPI * u1;
        double st = sin(theta);
        double sx = st * cos(phi), sy = st * sin(phi), sz = cos(theta);
        double sxy = sqrt(old[0] * old[0] + old[1] * old[1]);
        double cphi = 1.0, sphi = 0.0;
        if (sxy > OR_EPS8) { cphi = old[0] / sxy; sphi = old[1] / sxy; }
        double nrm = sqrt(old[0] * old[0] + old[1] * old[1] + old[2] * old[2]);
        double on[3] = {old[0] / nrm, old[1] / nrm, old[2] / nrm};
        out[0] = mag * (cphi * on[2] * sx - sphi * sy + on[0] * sz);
        out[1] = mag * (sphi * on[2] * sx + cphi * sy + on[1] * sz);
        out[2] = mag * (-sqrt(on[0] * on[0] + on[1] * on[1]) * sx + on[2] * sz);
    }
}

int64_t or_colour_pass_philox(const or_ham *h, const int32_t *colour, int c,
                              double beta, double *s, int replica,
                              uint64_t sweep, uint64_t seed, int mode, double tilt,
                              double *energy, int8_t *accept_out, double *de_out)
{
    int64_t rej = 0;
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    for (int i = 0; i < h->n; ++i) {
        if (colour[i] != c) { if (accept_out) accept_out[i] = -1; continue; }
        uint32_t ctr[4] = {(uint32_t)i, (uint32_t)replica, (uint32_t)sweep, (uint32_t)(sweep >> 32)};
        uint32_t x[4];
        or_philox4x32_10(ctr, key, x);
        double old[3] = {s[3 * i], s[3 * i + 1], s[3 * i + 2]};
        double nw[3];
        or_trial_spin(old, h->mag[i], mode, tilt, x, nw);
        s[3 * i] = nw[0]; s[3 * i + 1] = nw[1]; s[3 * i + 2] = nw[2];
        double ds[3] = {nw[0] - old[0], nw[1] - old[1], nw[2] - old[2]};
        double de = or_delta_energy(h, i, s, ds);
        if (de_out) de_out[i] = de;
        int acc = 1;
        if (de > 0.0) {
            double fac = exp(-beta * de);
            if (!(fac >= u24(x[2]))) acc = 0;
        }
        if (acc) { if (energy) *energy += de; }
        else { s[3 * i] = old[0]; s[3 * i + 1] = old[1]; s[3 * i + 2] = old[2]; rej++; }
        if (accept_out) accept_out[i] = (int8_t)acc;
    }
    return rej;
}

/* ------------------------------------------------------------------------ */
/* Supercell pair expansion to ELL (jij.F90:196-318 + 394-446).              */
/*                                                                           */
/* pairs: npairs rows of f1[3], f2[3] (fractional) and a value of vdim       */
/* components (1 for J and B, 3 for D = d * unit vector).  Atoms are given    */
/* species-major (the order param_get_atoms_moments leaves them in).          */
/* Output ELL arrays must hold n*npairs entries (the Fortran work arrays'     */
/* size); on return nn[i] and the compacted, site-fastest tables with stride  */
/* n are filled and *maxnb_out holds maxval(nn).  Returns 0, or -(row+1) for  */
/* an unrecognised first-atom position, -(npairs+row+1) for a second-atom one.*/
/* ------------------------------------------------------------------------ */
static int find_atom(const double *pos, int num_atoms, const double *atoms_frac)
{
    for (int a = 0; a < num_atoms; ++a)
        if (fabs(pos[0] - atoms_frac[3 * a]) <= OR_EPS4 &&
            fabs(pos[1] - atoms_frac[3 * a + 1]) <= OR_EPS4 &&
            fabs(pos[2] - atoms_frac[3 * a + 2]) <= OR_EPS4)
            return a;
    return -1;
}

static inline double snap(double x)
{
    double r = (double)lround(x);
    return (fabs(x - r) < OR_EPS5) ? r : x;
}

static inline long fmod_pos(long l, long L) { return ((l + 10 * L) % L); }

int or_build_ell(int num_atoms, const double *atoms_frac, const double *mag_cell,
                 const int32_t *sc, int open_boundary, int npairs,
                 const double *f1, const double *f2, const double *vals, int vdim,
                 int32_t *nn, int32_t *nb, double *val, int32_t *maxnb_out)
{
    const long L0 = sc[0], L1 = sc[1], L2 = sc[2];
    const long ncell = L0 * L1 * L2;
    const long n = ncell * num_atoms;
    int32_t *tot_nb = (int32_t *)calloc((size_t)n * npairs, sizeof(int32_t));
    double *tot_val = (double *)calloc((size_t)n * npairs * vdim, sizeof(double));
    int32_t *num = (int32_t *)calloc((size_t)n, sizeof(int32_t));
    int rc = 0;
    for (long cell = 0; cell < ncell && rc == 0; ++cell) {
        long lmn[3] = {cell % L0, (cell / L0) % L1, cell / (L0 * L1)};
        for (int p = 0; p < npairs; ++p) {
            double a1[3], a2[3], pos[3];
            long l[3];
            for (int c = 0; c < 3; ++c) a1[c] = snap(f1[3 * p + c] + (double)lmn[c]);
            for (int c = 0; c < 3; ++c) { l[c] = (long)floor(a1[c]); pos[c] = a1[c] - (double)l[c]; }
            long cell1 = fmod_pos(l[2], L2) * L1 * L0 + fmod_pos(l[1], L1) * L0 + fmod_pos(l[0], L0);
            int at1 = find_atom(pos, num_atoms, atoms_frac);
            if (at1 < 0) { rc = -(p + 1); break; }
            long i1 = cell1 * num_atoms + at1;
            num[i1] += 1;
            for (int c = 0; c < 3; ++c) a2[c] = snap(f2[3 * p + c] + (double)lmn[c]);
            for (int c = 0; c < 3; ++c) l[c] = (long)floor(a2[c]);
            if (open_boundary &&
                (l[0] < 0 || l[0] == L0 || l[1] < 0 || l[1] == L1 || l[2] < 0 || l[2] == L2))
                continue;
            for (int c = 0; c < 3; ++c) pos[c] = a2[c] - (double)l[c];
            long cell2 = fmod_pos(l[2], L2) * L1 * L0 + fmod_pos(l[1], L1) * L0 + fmod_pos(l[0], L0);
            int at2 = find_atom(pos, num_atoms, atoms_frac);
            if (at2 < 0) { rc = -(npairs + p + 1); break; }
            long i2 = cell2 * num_atoms + at2;
            long slot = (long)(num[i1] - 1) * n + i1;
            double mm = fabs(mag_cell[at1] * mag_cell[at2]);
            for (int c = 0; c < vdim; ++c) tot_val[slot * vdim + c] = vals[p * vdim + c] / mm;
            tot_nb[slot] = (int32_t)i2;
        }
    }
    int32_t maxnb = 0;
    if (rc == 0) {
        for (long i = 0; i < n; ++i) {
            int cnt = 0;
            for (int k = 0; k < npairs; ++k) {
                long slot = (long)k * n + i;
                int nz = 0;
                for (int c = 0; c < vdim; ++c) if (tot_val[slot * vdim + c] != 0.0) nz = 1;
                if (nz) {
                    long dst = (long)cnt * n + i;
                    nb[dst] = tot_nb[slot];
                    for (int c = 0; c < vdim; ++c) val[dst * vdim + c] = tot_val[slot * vdim + c];
                    cnt++;
                }
            }
            nn[i] = cnt;
            if (cnt > maxnb) maxnb = cnt;
        }
    }
    *maxnb_out = maxnb;
    free(tot_nb); free(tot_val); free(num);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* CPU baseline: the reference's PT main phase on host threads.             */
/*                                                                          */
/* Temperatures are block-split over threads as comms_array_split does      */
/* (comms.F90:153-176, one thread standing for one MPI rank); each thread   */
/* runs pt_steps_swap typewriter sweeps of its temperatures with its own    */
/* MT19937 stream, measuring after every steps_measure sweeps               */
/* (pt.F90:773-864: E accumulators, magnetization_get, Pm_get), then thread */
/* 0 performs pt_swap.  Returns the number of site updates done; with       */
/* seconds != NULL also the wall time of the swap intervals alone (from the */
/* barrier all threads reach after their set-up to the last one), without   */
/* the initial energies and the thread start-up.                            */
/* ------------------------------------------------------------------------ */
#include <pthread.h>
#include <time.h>

typedef struct {
    const or_ham *h;
    int R, nthreads, tid, mode;
    double tilt;
    const double *tems;
    double *spins, *e2, *data, *pm;
    int64_t *rejected, *num_swaps;
    int32_t *map;
    int64_t n_swap_intervals, pss, steps_measure;
    int32_t seed;
    pthread_barrier_t *bar;
    double *tmp;
    or_mt root_mt;
    int64_t updates;
    double t_start, t_end;
} or_bench_ctx;

static double or_now(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static void *or_bench_worker(void *arg)
{
    or_bench_ctx *c = (or_bench_ctx *)arg;
    const or_ham *h = c->h;
    const int n = h->n;
    int base = c->R / c->nthreads, rem = c->R % c->nthreads;
    int t0 = c->tid * base + (c->tid < rem ? c->tid : rem);
    int t1 = t0 + base + (c->tid < rem ? 1 : 0);
    int nf = or_num_freq(h);
    or_mt mt;
    or_mt_init(&mt, c->seed + c->tid);
    c->updates = 0;
    pthread_barrier_wait(c->bar);
    if (c->tid == 0) c->t_start = or_now();
    for (int64_t lsw = 1; lsw <= c->n_swap_intervals; ++lsw) {
        for (int t = t0; t < t1; ++t) {
            double beta = 1.0 / c->tems[t];
            double *s = c->spins + (size_t)3 * n * t;
            for (int64_t mc = 0; mc < c->pss; ++mc) {
                for (int64_t ms = 0; ms < c->steps_measure; ++ms)
                    for (int i = 0; i < n; ++i)
                        or_metropolis(h, &mt, i, beta, s, &c->e2[t], &c->rejected[t], c->mode, c->tilt);
                c->updates += (int64_t)n * c->steps_measure;
                double e = c->e2[t], ee = e * e, *d = c->data + 6 * t;
                d[0] += e; d[1] += ee; d[2] += ee * ee;
                double m2 = or_magnetization2(h, s);
                d[3] += sqrt(m2); d[4] += m2; d[5] += m2 * m2;
                or_pm(h, s, nf, c->pm + (size_t)nf * t);
            }
        }
        pthread_barrier_wait(c->bar);
        if (c->tid == 0)
            or_pt_swap((int)((lsw + 1) % 2) + 1, c->R, c->tems, n, c->spins, c->e2, c->map, c->num_swaps,
                       &c->root_mt, c->tmp);
        pthread_barrier_wait(c->bar);
    }
    if (c->tid == 0) c->t_end = or_now();
    return NULL;
}

int64_t or_pt_bench(const or_ham *h, int nthreads, int R, const double *tems, double *spins,
                    int64_t n_swap_intervals, int64_t pss, int64_t steps_measure, int mode,
                    double tilt, int32_t seed, double *seconds)
{
    if (nthreads > R) nthreads = R;
    if (nthreads < 1) nthreads = 1;
    const int n = h->n;
    int nf = or_num_freq(h);
    double *e2 = (double *)calloc((size_t)R, sizeof(double));
    double *data = (double *)calloc((size_t)6 * R, sizeof(double));
    double *pm = (double *)calloc((size_t)nf * R, sizeof(double));
    int64_t *rej = (int64_t *)calloc((size_t)R, sizeof(int64_t));
    int64_t *sw = (int64_t *)calloc((size_t)2 * R, sizeof(int64_t));
    int32_t *map = (int32_t *)malloc(sizeof(int32_t) * R);
    double *tmp = (double *)malloc(sizeof(double) * 3 * (size_t)n);
    for (int t = 0; t < R; ++t) { map[t] = t + 1; e2[t] = or_energy(h, spins + (size_t)3 * n * t); }
    pthread_barrier_t bar;
    pthread_barrier_init(&bar, NULL, (unsigned)nthreads);
    or_bench_ctx *ctx = (or_bench_ctx *)calloc((size_t)nthreads, sizeof(or_bench_ctx));
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
    for (int k = 0; k < nthreads; ++k) {
        or_bench_ctx *c = &ctx[k];
        c->h = h; c->R = R; c->nthreads = nthreads; c->tid = k; c->mode = mode; c->tilt = tilt;
        c->tems = tems; c->spins = spins; c->e2 = e2; c->data = data; c->pm = pm;
        c->rejected = rej; c->num_swaps = sw; c->map = map;
        c->n_swap_intervals = n_swap_intervals; c->pss = pss; c->steps_measure = steps_measure;
        c->seed = seed; c->bar = &bar; c->tmp = tmp;
        if (k == 0) or_mt_init(&c->root_mt, seed - 1);
        pthread_create(&th[k], NULL, or_bench_worker, c);
    }
    int64_t total = 0;
    for (int k = 0; k < nthreads; ++k) { pthread_join(th[k], NULL); total += ctx[k].updates; }
    if (seconds) *seconds = ctx[0].t_end - ctx[0].t_start;
    pthread_barrier_destroy(&bar);
    free(ctx); free(th); free(e2); free(data); free(pm); free(rej); free(sw); free(map); free(tmp);
    return total;
}
