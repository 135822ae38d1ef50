// Learned proposal: network sizes, the von Mises-Fisher mixture head, its
// sampler, its exact log-density on the unit sphere and the gradient of that
// log-density with respect to the network outputs.
//
// The proposal for the spin of site i is a mixture of kComp vMF densities
//   q(s) = sum_k w_k C(kappa_k) exp(kappa_k mu_k . s),
//   C(kappa) = kappa / (4 pi sinh kappa),
//   log C(kappa) = log kappa - log 2pi - kappa - log1p(-exp(-2 kappa)),
// whose parameters come from an MLP of the site's environment only (its
// linear field g, quadratic form Q and beta), never from s_i itself.  One
// evaluation therefore gives q for the current and the proposed spin, and the
// Metropolis-Hastings test
//   accept if  u < exp(-beta dE) q(s_old) / q(s_new)
// is exact (detailed balance holds for any network weights).
//
// Everything is expressed in a local frame (e1, e2, e3) built from the
// environment: e3 = -g/|g| (the direction the linear term favours), e1 the
// single-ion axis (or x) made orthogonal to e3.  The output parametrisation
// is residual around the exact conditional of a pure Heisenberg site,
// vMF(e3, kappa0 = beta m |g|): with zero outputs every component is that
// density, and the network learns the corrections that the biquadratic and
// single-ion terms need.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace esp {

constexpr int kMlpIn = 12;    // features
constexpr int kMlpInPad = 16; // padded to the MMA k-step
constexpr int kMlpHid = 128;
constexpr int kComp = 4;
constexpr int kMlpOut = 5 * kComp;  // per component: direction (3), kappa (1), logit (1)
constexpr int kMlpOutPad = 32;
// logical parameter count: W1[128][12] b1 W2[128][128] b2 W3[20][128] b3
constexpr int kLpParams = kMlpHid * kMlpIn + kMlpHid + kMlpHid * kMlpHid + kMlpHid + kMlpOut * kMlpHid + kMlpOut;
constexpr float kKappaMin = 1e-3f, kKappaMax = 1e4f;

struct VmfMix {
    float mu[kComp][3];   // unit mean directions (local frame)
    float vn[kComp];      // |raw direction| (for the gradient)
    float kappa[kComp];
    float logw[kComp];    // log of the normalised mixture weights
    float dkappa[kComp];  // d kappa / d raw output (0 where clamped)
};

__host__ __device__ __forceinline__ float softplusf_(float x) { return x > 20.f ? x : log1pf(expf(x)); }
__host__ __device__ __forceinline__ float sigmoidf_(float x) { return 1.f / (1.f + expf(-x)); }
// inverse of softplus, argument floored at 1e-4
__host__ __device__ __forceinline__ float softplus_invf_(float y)
{
    y = fmaxf(y, 1e-4f);
    return y > 20.f ? y + log1pf(-expf(-y)) : logf(expm1f(y));
}

// Raw network outputs o[0..19] -> mixture parameters.  Per component k:
// direction v = (o[5k], o[5k+1], 1 + o[5k+2]), mu = v/|v|;
// kappa = clamp(softplus(o[5k+3] + softplus^-1(kappa0)), 1e-3, 1e4), which is
// kappa0 itself for a zero output; weight logit o[5k+4].
__host__ __device__ __forceinline__ void vmf_params(const float *o, float kappa0, VmfMix &m)
{
    const float k0i = softplus_invf_(kappa0);
    float lmax = -1e30f;
#pragma unroll
    for (int k = 0; k < kComp; ++k) lmax = fmaxf(lmax, o[5 * k + 4]);
    float z = 0.f;
#pragma unroll
    for (int k = 0; k < kComp; ++k) z += expf(o[5 * k + 4] - lmax);
    const float lz = lmax + logf(z);
#pragma unroll
    for (int k = 0; k < kComp; ++k) {
        const float x = o[5 * k], y = o[5 * k + 1], w = 1.f + o[5 * k + 2];
        const float n = sqrtf(x * x + y * y + w * w) + 1e-12f;
        m.vn[k] = n;
        m.mu[k][0] = x / n; m.mu[k][1] = y / n; m.mu[k][2] = w / n;
        const float pre = o[5 * k + 3] + k0i;
        const float kap = softplusf_(pre);
        m.kappa[k] = fminf(fmaxf(kap, kKappaMin), kKappaMax);
        m.dkappa[k] = (kap > kKappaMin && kap < kKappaMax) ? sigmoidf_(pre) : 0.f;
        m.logw[k] = o[5 * k + 4] - lz;
    }
}

// log C(kappa) = log(kappa / (4 pi sinh kappa)), stable for all kappa > 0.
__host__ __device__ __forceinline__ float vmf_logc(float kappa)
{
    return logf(kappa) - 1.8378770664093453f /* log 2 pi */ - kappa - log1pf(-expf(-2.f * kappa));
}

// d log C / d kappa = 1/kappa - coth(kappa), series below 1e-2.
__host__ __device__ __forceinline__ float vmf_dlogc(float kappa)
{
    if (kappa < 1e-2f) return kappa * (-1.f / 3.f + kappa * kappa * (1.f / 45.f));
    return 1.f / kappa - 1.f - 2.f / expm1f(2.f * kappa);
}

// log q(s) for a unit vector s (local frame); t[] receives the per-component
// log terms when non-null.
__host__ __device__ __forceinline__ float vmf_logpdf(const VmfMix &m, float sx, float sy, float sz, float *t_out = nullptr)
{
    float t[kComp], tmax = -1e30f;
#pragma unroll
    for (int k = 0; k < kComp; ++k) {
        t[k] = m.logw[k] + vmf_logc(m.kappa[k]) + m.kappa[k] * (m.mu[k][0] * sx + m.mu[k][1] * sy + m.mu[k][2] * sz);
        tmax = fmaxf(tmax, t[k]);
    }
    float acc = 0.f;
#pragma unroll
    for (int k = 0; k < kComp; ++k) acc += expf(t[k] - tmax);
    const float lq = tmax + logf(acc);
    if (t_out)
#pragma unroll
        for (int k = 0; k < kComp; ++k) t_out[k] = t[k];
    return lq;
}

// d log q(s) / d o for the 20 raw outputs (o as in vmf_params).
__host__ __device__ __forceinline__ float vmf_logpdf_grad(const VmfMix &m, float sx, float sy, float sz, float *d)
{
    float t[kComp];
    const float lq = vmf_logpdf(m, sx, sy, sz, t);
    for (int k = 0; k < kComp; ++k) {
        const float r = expf(t[k] - lq);           // responsibility
        const float w = expf(m.logw[k]);
        const float c = m.mu[k][0] * sx + m.mu[k][1] * sy + m.mu[k][2] * sz;
        const float g = r * m.kappa[k] / m.vn[k];   // d lq / d v = g (s - c mu)
        d[5 * k] = g * (sx - c * m.mu[k][0]);
        d[5 * k + 1] = g * (sy - c * m.mu[k][1]);
        d[5 * k + 2] = g * (sz - c * m.mu[k][2]);
        d[5 * k + 3] = r * (vmf_dlogc(m.kappa[k]) + c) * m.dkappa[k];
        d[5 * k + 4] = r - w;
    }
    return lq;
}

// Draw a unit vector (local frame) from the mixture with three uniforms in
// [0,1): u0 picks the component, u1 the cosine to its mean by the exact
// inverse CDF on S^2, t = 1 + log1p((1 - u1) expm1(-2 kappa)) / kappa, u2 the
// azimuth around the mean.
__host__ __device__ __forceinline__ void vmf_sample(const VmfMix &m, float u0, float u1, float u2, float &sx,
                                                    float &sy, float &sz)
{
    // component choice by selection (no dynamic indexing: stays in registers)
    float kap = m.kappa[kComp - 1];
    float mx = m.mu[kComp - 1][0], my = m.mu[kComp - 1][1], mz = m.mu[kComp - 1][2];
    float c = 0.f;
    bool found = false;
#pragma unroll
    for (int j = 0; j < kComp - 1; ++j) {
        c += expf(m.logw[j]);
        if (!found && u0 < c) {
            found = true;
            kap = m.kappa[j]; mx = m.mu[j][0]; my = m.mu[j][1]; mz = m.mu[j][2];
        }
    }
    float t = 1.f + log1pf((1.f - u1) * expm1f(-2.f * kap)) / kap;
    t = fminf(fmaxf(t, -1.f), 1.f);
    const float r = sqrtf(fmaxf(0.f, 1.f - t * t));
    // orthonormal e1, e2 perpendicular to mu
    float ax = 1.f, ay = 0.f;
    if (fabsf(mx) > 0.9f) { ax = 0.f; ay = 1.f; }
    // e1 = a x mu with a = (ax, ay, 0)
    float e1x = ay * mz, e1y = -ax * mz, e1z = ax * my - ay * mx;
    const float n1 = 1.f / sqrtf(e1x * e1x + e1y * e1y + e1z * e1z);
    e1x *= n1; e1y *= n1; e1z *= n1;
    const float e2x = my * e1z - mz * e1y, e2y = mz * e1x - mx * e1z, e2z = mx * e1y - my * e1x;
    float sp, cp;
#ifdef __CUDA_ARCH__
    sincospif(2.f * u2, &sp, &cp);
#else
    sp = sinf(6.283185307179586f * u2); cp = cosf(6.283185307179586f * u2);
#endif
    sx = t * mx + r * (cp * e1x + sp * e2x);
    sy = t * my + r * (cp * e1y + sp * e2y);
    sz = t * mz + r * (cp * e1z + sp * e2z);
    const float nn = 1.f / sqrtf(sx * sx + sy * sy + sz * sz);
    sx *= nn; sy *= nn; sz *= nn;
}

// Local frame and features of a site.  Inputs: beta, spin length mag, the
// linear field g (E_i(s) = g.s + s^T Q s for the spin vector s), Q as
// (xx, yy, zz, xy, xz, yz), and a reference axis (the single-ion axis, or x).
// Outputs: the frame rows e[0..2] (global components), kappa0 = beta mag |g|
// and the 12 features
//   log1p(kappa0), kappa0/20, beta mag^2 Q_local (6), beta mag^2 tr Q,
//   beta mag^2 (Q_zz - (Q_xx + Q_yy)/2)_local, log(beta), 1/(1 + kappa0).
struct LpFrame {
    float e[3][3];
    float kappa0;
};

__host__ __device__ __forceinline__ void lp_frame_features(float beta, float mag, float gx, float gy, float gz,
                                                           const float q[6], float ax, float ay, float az,
                                                           LpFrame &fr, float *f)
{
    const float gn = sqrtf(gx * gx + gy * gy + gz * gz);
    const float kappa0 = beta * mag * gn;
    float e3x = 0.f, e3y = 0.f, e3z = 1.f;
    if (kappa0 > 1e-6f) { e3x = -gx / gn; e3y = -gy / gn; e3z = -gz / gn; }
    // e1: the reference axis without its e3 part; x or y when it is (nearly) parallel
    float d = ax * e3x + ay * e3y + az * e3z;
    float e1x = ax - d * e3x, e1y = ay - d * e3y, e1z = az - d * e3z;
    float n1 = e1x * e1x + e1y * e1y + e1z * e1z;
    if (n1 < 1e-6f) {
        const float bx = fabsf(e3x) < 0.9f ? 1.f : 0.f, by = 1.f - bx;
        d = bx * e3x + by * e3y;
        e1x = bx - d * e3x; e1y = by - d * e3y; e1z = -d * e3z;
        n1 = e1x * e1x + e1y * e1y + e1z * e1z;
    }
    n1 = 1.f / sqrtf(n1);
    e1x *= n1; e1y *= n1; e1z *= n1;
    const float e2x = e3y * e1z - e3z * e1y, e2y = e3z * e1x - e3x * e1z, e2z = e3x * e1y - e3y * e1x;
    fr.e[0][0] = e1x; fr.e[0][1] = e1y; fr.e[0][2] = e1z;
    fr.e[1][0] = e2x; fr.e[1][1] = e2y; fr.e[1][2] = e2z;
    fr.e[2][0] = e3x; fr.e[2][1] = e3y; fr.e[2][2] = e3z;
    fr.kappa0 = kappa0;
    // Q in the local frame: L_ab = e_a^T Q e_b
    const float sc = beta * mag * mag;
    float ql[6];
    {
        float qe[3][3];
        for (int a = 0; a < 3; ++a) {
            const float vx = fr.e[a][0], vy = fr.e[a][1], vz = fr.e[a][2];
            qe[a][0] = q[0] * vx + q[3] * vy + q[4] * vz;
            qe[a][1] = q[3] * vx + q[1] * vy + q[5] * vz;
            qe[a][2] = q[4] * vx + q[5] * vy + q[2] * vz;
        }
        auto dot = [&](int a, int b) {
            return fr.e[b][0] * qe[a][0] + fr.e[b][1] * qe[a][1] + fr.e[b][2] * qe[a][2];
        };
        ql[0] = dot(0, 0); ql[1] = dot(1, 1); ql[2] = dot(2, 2);
        ql[3] = dot(0, 1); ql[4] = dot(0, 2); ql[5] = dot(1, 2);
    }
    f[0] = log1pf(kappa0);
    f[1] = 0.05f * kappa0;
    for (int i = 0; i < 6; ++i) f[2 + i] = sc * ql[i];
    f[8] = sc * (ql[0] + ql[1] + ql[2]);
    f[9] = sc * (ql[2] - 0.5f * (ql[0] + ql[1]));
    f[10] = logf(beta);
    f[11] = 1.f / (1.f + kappa0);
}

}  // namespace esp
