// Device-side building blocks shared by the Monte Carlo kernels.
//
// Random numbers: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), a
// counter-based generator, replaces the reference's per-rank MT19937 stream
// (ESpinS src/mtprng.f90).  One call yields the three uniforms one
// Metropolis trial needs (get_quant.F90:80-93 draws two for the trial spin
// and a third for the acceptance test only when dE > 0).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace esp {

struct Philox4 {
    uint32_t x, y, z, w;
};

__host__ __device__ __forceinline__ uint32_t mulhi32(uint32_t a, uint32_t b)
{
#ifdef __CUDA_ARCH__
    return __umulhi(a, b);
#else
    return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

// Ten rounds; the key is bumped by the Weyl constants before rounds 2..10.
__host__ __device__ __forceinline__ Philox4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                                          uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        const uint32_t hi0 = mulhi32(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        const uint32_t hi1 = mulhi32(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    }
    return Philox4{c0, c1, c2, c3};
}

// Uniform in [0,1) with 24 bits: exact in float and in double.
__host__ __device__ __forceinline__ float u24f(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }
// Uniform in [0,1) with 53 bits for FP64 decisions (PT swaps).
__host__ __device__ __forceinline__ double u53(uint32_t a, uint32_t b)
{
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

// Every sweep kernel evaluates the trial, the local field and the energy
// change through the functions below, written without implicit contraction
// (explicit fmaf / __fmul_rn / __fadd_rn), so all kernels round the same way
// and follow the same trajectory from the same state.

// Trial spin of metropolis (get_quant.F90:80-162) in FP32.
//  mode 0 'random': cos(theta) = 2u0-1, phi = 2 pi u1, length |mag|
//  mode 1 'const' : theta = tilt*acos(2u0-1) about the old direction,
//                   rotated as M = Rz(phi0) Ry(theta0) (get_quant.F90:136-159)
__device__ __forceinline__ void trial_spin(int mode, float tilt, float mag, float ox, float oy, float oz,
                                           uint32_t x0, uint32_t x1, float &nx, float &ny, float &nz)
{
    const float u0 = u24f(x0), u1 = u24f(x1);
    // phi = 2 pi u1 = psi + pi with psi = 2 pi (u1 - 1/2) in [-pi, pi), where
    // the hardware sine and cosine are accurate to ~4e-7 (u1 - 1/2 is exact)
    float sphi, cphi;
    {
        float sp, cp;
        __sincosf(__fmul_rn(6.28318530717958648f, u1 - 0.5f), &sp, &cp);
        sphi = -sp;
        cphi = -cp;
    }
    const float c = fmaf(2.0f, u0, -1.0f);   // exact: u0 has 24 bits
    if (mode == 0) {
        const float s = sqrtf(fmaxf(0.0f, fmaf(-c, c, 1.0f)));
        const float ms = __fmul_rn(mag, s);
        nx = __fmul_rn(ms, cphi);
        ny = __fmul_rn(ms, sphi);
        nz = __fmul_rn(mag, c);
    } else {
        const float theta = __fmul_rn(tilt, acosf(c));
        float st, ct;
        __sincosf(theta, &st, &ct);   // theta in [0, pi]
        const float tx = __fmul_rn(st, cphi), ty = __fmul_rn(st, sphi), tz = ct;
        const float sxy = sqrtf(fmaf(oy, oy, __fmul_rn(ox, ox)));
        float c0 = 1.0f, s0 = 0.0f;
        if (sxy > 1e-8f) { c0 = ox / sxy; s0 = oy / sxy; }
        const float inv = rsqrtf(fmaf(oz, oz, fmaf(oy, oy, __fmul_rn(ox, ox))));
        const float ax = __fmul_rn(ox, inv), ay = __fmul_rn(oy, inv), az = __fmul_rn(oz, inv);
        nx = __fmul_rn(mag, fmaf(ax, tz, fmaf(-s0, ty, __fmul_rn(__fmul_rn(c0, az), tx))));
        ny = __fmul_rn(mag, fmaf(ay, tz, fmaf(c0, ty, __fmul_rn(__fmul_rn(s0, az), tx))));
        nz = __fmul_rn(mag, fmaf(az, tz, __fmul_rn(-sqrtf(fmaf(ay, ay, __fmul_rn(ax, ax))), tx)));
    }
}

// The Boltzmann test of metropolis (get_quant.F90:166-178): accept a move
// with energy change de when de <= 0, else when exp(-beta de) >= u (the
// third uniform).  The hardware exponential is within a few parts in 1e6 of
// exp, which moves only decisions where exp(-beta de) lies that close to u.
__device__ __forceinline__ bool metropolis_accept(float beta, float de, uint32_t u_bits)
{
    return !(de > 0.0f) || __expf(-beta * de) >= u24f(u_bits);
}

// DM share of one neighbour in the local field, g += s_k x D_ik
// (delta_energy_get, get_quant.F90:327-333)
__device__ __forceinline__ void dm_field(float dx, float dy, float dz, float tx, float ty, float tz, float &gx,
                                         float &gy, float &gz)
{
    gx = fmaf(tz, -dy, fmaf(ty, dz, gx));
    gy = fmaf(tx, -dz, fmaf(tz, dx, gy));
    gz = fmaf(ty, -dx, fmaf(tx, dy, gz));
}

// Biquadratic share of one neighbour in the quadratic form Q (get_quant.F90:316-325)
__device__ __forceinline__ void bq_form(float Bv, float tx, float ty, float tz, float &qxx, float &qyy, float &qzz,
                                        float &qxy, float &qxz, float &qyz)
{
    const float bx = __fmul_rn(Bv, tx), by = __fmul_rn(Bv, ty), bz = __fmul_rn(Bv, tz);
    qxx = fmaf(bx, tx, qxx); qyy = fmaf(by, ty, qyy); qzz = fmaf(bz, tz, qzz);
    qxy = fmaf(bx, ty, qxy); qxz = fmaf(bx, tz, qxz); qyz = fmaf(by, tz, qyz);
}

// Single-ion share of Q: Delta a a^T (get_quant.F90:306-314); s = (a, Delta)
__device__ __forceinline__ void si_form(float4 s, float &qxx, float &qyy, float &qzz, float &qxy, float &qxz,
                                        float &qyz)
{
    const float dx = __fmul_rn(s.w, s.x), dy = __fmul_rn(s.w, s.y), dz = __fmul_rn(s.w, s.z);
    qxx = fmaf(dx, s.x, qxx); qyy = fmaf(dy, s.y, qyy); qzz = fmaf(dz, s.z, qzz);
    qxy = fmaf(dx, s.y, qxy); qxz = fmaf(dx, s.z, qxz); qyz = fmaf(dy, s.z, qyz);
}

// Energy change of s_old -> s_new with local field g and quadratic form Q:
// g.d + d^T Q (s_new + s_old), d = s_new - s_old (the local form of
// delta_energy_get); quad = false skips the Q term
__device__ __forceinline__ float delta_energy(bool quad, float gx, float gy, float gz, float qxx, float qyy, float qzz,
                                              float qxy, float qxz, float qyz, float ox, float oy, float oz, float nx,
                                              float ny, float nz)
{
    const float dx = __fsub_rn(nx, ox), dy = __fsub_rn(ny, oy), dz = __fsub_rn(nz, oz);
    float de = fmaf(gz, dz, fmaf(gy, dy, __fmul_rn(gx, dx)));
    if (quad) {
        const float px = __fadd_rn(nx, ox), py = __fadd_rn(ny, oy), pz = __fadd_rn(nz, oz);
        const float ax = fmaf(qxz, pz, fmaf(qxy, py, __fmul_rn(qxx, px)));
        const float ay = fmaf(qyz, pz, fmaf(qyy, py, __fmul_rn(qxy, px)));
        const float az = fmaf(qzz, pz, fmaf(qyz, py, __fmul_rn(qxz, px)));
        de = fmaf(dz, az, fmaf(dy, ay, fmaf(dx, ax, de)));
    }
    return de;
}

// Bin of a unit cell's value m on the P(M) grid of Pm_get
// (get_quant.F90:425-493): max(nint((m - m_min) / (m_max - m_min) * (nf-1)) + 1, 1),
// clamped to nf; FP32 (an edge flip needs m within ~1e-7 of a bin edge).
// scale = (nf - 1) / (m_max - m_min).  Returns the 1-based bin.  m is |sum s|
// for P(M) and P(SM), the signed sum of s.a for P(OP).
// Unevaluated sums hi + lo of two floats (Knuth's two-sum, Dekker's
// normalisation): sums of FP32 terms kept to about 2^-46 relative without the
// FP64 pipe.
struct F2 {
    float hi, lo;
};

__device__ __forceinline__ F2 f2_add(F2 x, F2 y)
{
    const float s = __fadd_rn(x.hi, y.hi);
    const float bb = __fsub_rn(s, x.hi);
    float e = __fadd_rn(__fsub_rn(x.hi, __fsub_rn(s, bb)), __fsub_rn(y.hi, bb));
    e = __fadd_rn(e, __fadd_rn(x.lo, y.lo));
    const float h = __fadd_rn(s, e);
    return F2{h, __fsub_rn(e, __fsub_rn(h, s))};
}

__device__ __forceinline__ F2 f2_add(F2 x, float y) { return f2_add(x, F2{y, 0.f}); }

__device__ __forceinline__ F2 f2_shfl_down(F2 x, int o)
{
    return F2{__shfl_down_sync(0xffffffffu, x.hi, o), __shfl_down_sync(0xffffffffu, x.lo, o)};
}

__device__ __forceinline__ double f2_to_double(F2 x) { return (double)x.hi + (double)x.lo; }

// Adds one spin's s.a to op and c s to (qx, qy, qz), w = (a, c), with
// explicitly rounded fused multiply-adds: every kernel that measures the order
// parameter or the staggered magnetisation gets the same bits for a cell.
__device__ __forceinline__ void obs_add(float ox, float oy, float oz, float4 w, float &op, float &qx, float &qy,
                                        float &qz)
{
    op = __fmaf_rn(oz, w.z, __fmaf_rn(oy, w.y, __fmaf_rn(ox, w.x, op)));
    qx = __fmaf_rn(w.w, ox, qx);
    qy = __fmaf_rn(w.w, oy, qy);
    qz = __fmaf_rn(w.w, oz, qz);
}

__device__ __forceinline__ int pm_bin_value(float m, float m_min, float scale, int nf)
{
    int bin = (int)floorf((m - m_min) * scale + 0.5f) + 1;  // nint of a non-negative value
    bin = bin < 1 ? 1 : bin;
    return bin > nf ? nf : bin;
}

__device__ __forceinline__ int pm_bin(float mx, float my, float mz, float m_min, float scale, int nf)
{
    return pm_bin_value(sqrtf(mx * mx + my * my + mz * mz), m_min, scale, nf);
}

// Division by an invariant integer d >= 1 as a multiply-high, an add and a
// shift (T. Granlund, P. Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994): with l = ceil(log2 d) and
// m = floor(2^32 (2^l - d) / d) + 1, n / d = (mulhi(n, m) + n) >> l for
// 0 <= n < 2^31.
struct FastDiv {
    uint32_t d, m, s;
};

inline FastDiv make_fastdiv(uint32_t d)
{
    FastDiv f{d, 0u, 0u};
    uint32_t l = 0;
    while ((1ull << l) < d) ++l;
    f.s = l;
    f.m = (uint32_t)((((1ull << l) - d) << 32) / d + 1ull);
    if (d == 1) f.m = 0u;
    return f;
}

__host__ __device__ __forceinline__ int fdiv(int n, const FastDiv &f)
{
    return (int)((mulhi32((uint32_t)n, f.m) + (uint32_t)n) >> f.s);
}

__host__ __device__ __forceinline__ void fdivmod(int n, const FastDiv &f, int &q, int &r)
{
    q = fdiv(n, f);
    r = n - q * (int)f.d;
}

// Arguments of the colour-class sweep over the merged ELL tables.
struct SweepArgs {
    // tables, permuted site order (colour-major); entry k of site p at k*N+p
    const int32_t *nnb;
    const int32_t *nbr;
    const float *J, *B, *Dx, *Dy, *Dz;
    const int32_t *perm;      // permuted -> reference site index (0-based)
    const float *mag;         // [N] permuted
    const float4 *si;         // [num_atoms] (ax, ay, az, Delta) or null
    const float4 *fld;        // [num_atoms] (f ax, f ay, f az, 0) or null
    // state, spin (p, r) at p*R + r
    float *sx, *sy, *sz;
    const int32_t *temp_of;   // replica -> temperature slot
    const float *beta;        // slot -> 1/T
    double *part;             // [blocks][slots][4]: dE, dMx, dMy, dMz of accepted moves
    unsigned long long *part_rej;   // [blocks][slots]: rejected trials
    int32_t slots;            // min(R, blockDim)
    int32_t N, R, num_atoms;
    int32_t off_c, n_c;       // colour class: permuted sites [off_c, off_c + n_c)
    int32_t mode;
    float tilt;
    uint32_t key0, key1, sw_lo, sw_hi;
    // device sweep counter added to (sw_hi, sw_lo), or null (replayed graphs
    // keep their launch arguments and advance the counter instead)
    const unsigned long long *ctr;
};

// The sweep index of a launch: the host value plus the device counter.
__device__ __forceinline__ void sweep_index(const SweepArgs &a, uint32_t &lo, uint32_t &hi)
{
    unsigned long long s = ((unsigned long long)a.sw_hi << 32) | a.sw_lo;
    if (a.ctr) s += *a.ctr;
    lo = (uint32_t)s;
    hi = (uint32_t)(s >> 32);
}

}  // namespace esp
