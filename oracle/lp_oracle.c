/*
 * lp_oracle.c -- FP64 CPU restatement of the learned proposal's network, its
 * von Mises-Fisher mixture head and the exact gradient of the training loss.
 *
 * TEST INFRASTRUCTURE ONLY: the checker of the GPU kernels in
 * espins_gb300/csrc/esp_learned.cu (forward pass, log-density, sampler and
 * backward pass).  Only tests/ may load it.  The learned proposal has no
 * counterpart in the reference, so this file follows the published
 * mathematics it uses:
 *   - the vMF density on S^2, C(k) = k / (4 pi sinh k) (Fisher 1953);
 *   - inverse-CDF sampling of the cosine to the mean direction,
 *     t = 1 + log(u + (1 - u) exp(-2k)) / k (Wood 1994);
 *   - reverse-mode differentiation of an MLP with ReLU activations.
 *
 * Network: h1 = relu(W1 x + b1), h2 = relu(W2 h1 + b2), o = W3 h2 + b3 with
 * 12 inputs, two hidden layers of 128 and 20 outputs.  Parameters in the
 * order W1[128][12] b1[128] W2[128][128] b2[128] W3[20][128] b3[20] (rows are
 * outputs).  Output k of the mixture (k = 0..3): direction (o[5k], o[5k+1],
 * 1 + o[5k+2]) normalised, concentration clamp(softplus(o[5k+3] +
 * softplus^-1(max(kappa0, 1e-4))), 1e-3, 1e4), weight softmax over o[5k+4].
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#define LP_IN 12
#define LP_HID 128
#define LP_OUT 20
#define LP_COMP 4
#define LP_NPARAM (LP_HID * LP_IN + LP_HID + LP_HID * LP_HID + LP_HID + LP_OUT * LP_HID + LP_OUT)
#define KAPPA_MIN 1e-3
#define KAPPA_MAX 1e4

int or_lp_num_params(void) { return LP_NPARAM; }

typedef struct {
    const double *w1, *b1, *w2, *b2, *w3, *b3;
} lp_net;

typedef struct {
    double *w1, *b1, *w2, *b2, *w3, *b3;
} lp_grad;

static lp_net net_of(const double *p)
{
    lp_net n;
    n.w1 = p; n.b1 = n.w1 + LP_HID * LP_IN;
    n.w2 = n.b1 + LP_HID; n.b2 = n.w2 + LP_HID * LP_HID;
    n.w3 = n.b2 + LP_HID; n.b3 = n.w3 + LP_OUT * LP_HID;
    return n;
}

static lp_grad grad_of(double *p)
{
    lp_grad n;
    n.w1 = p; n.b1 = n.w1 + LP_HID * LP_IN;
    n.w2 = n.b1 + LP_HID; n.b2 = n.w2 + LP_HID * LP_HID;
    n.w3 = n.b2 + LP_HID; n.b3 = n.w3 + LP_OUT * LP_HID;
    return n;
}

static void forward1(const lp_net *n, const double *x, double *h1, double *h2, double *o)
{
    for (int j = 0; j < LP_HID; ++j) {
        double a = n->b1[j];
        for (int k = 0; k < LP_IN; ++k) a += n->w1[j * LP_IN + k] * x[k];
        h1[j] = a > 0.0 ? a : 0.0;
    }
    for (int j = 0; j < LP_HID; ++j) {
        double a = n->b2[j];
        for (int k = 0; k < LP_HID; ++k) a += n->w2[j * LP_HID + k] * h1[k];
        h2[j] = a > 0.0 ? a : 0.0;
    }
    for (int j = 0; j < LP_OUT; ++j) {
        double a = n->b3[j];
        for (int k = 0; k < LP_HID; ++k) a += n->w3[j * LP_HID + k] * h2[k];
        o[j] = a;
    }
}

void or_lp_forward(const double *params, const double *x, int64_t n, double *out)
{
    lp_net net = net_of(params);
    double h1[LP_HID], h2[LP_HID];
    for (int64_t i = 0; i < n; ++i) forward1(&net, x + i * LP_IN, h1, h2, out + i * LP_OUT);
}

typedef struct {
    double mu[LP_COMP][3], vn[LP_COMP], kappa[LP_COMP], logw[LP_COMP], dkappa[LP_COMP];
} mix_t;

static double softplus(double x) { return x > 30.0 ? x : log1p(exp(x)); }

static double softplus_inv(double y)
{
    y = fmax(y, 1e-4);
    return y > 20.0 ? y + log1p(-exp(-y)) : log(expm1(y));
}

static void mix_params(const double *o, double kappa0, mix_t *m)
{
    const double k0i = softplus_inv(kappa0);
    double lmax = -1e300;
    for (int k = 0; k < LP_COMP; ++k) lmax = fmax(lmax, o[5 * k + 4]);
    double z = 0.0;
    for (int k = 0; k < LP_COMP; ++k) z += exp(o[5 * k + 4] - lmax);
    const double lz = lmax + log(z);
    for (int k = 0; k < LP_COMP; ++k) {
        const double x = o[5 * k], y = o[5 * k + 1], w = 1.0 + o[5 * k + 2];
        const double nv = sqrt(x * x + y * y + w * w);
        m->vn[k] = nv;
        m->mu[k][0] = x / nv; m->mu[k][1] = y / nv; m->mu[k][2] = w / nv;
        const double pre = o[5 * k + 3] + k0i;
        const double kap = softplus(pre);
        m->kappa[k] = fmin(fmax(kap, KAPPA_MIN), KAPPA_MAX);
        m->dkappa[k] = (kap > KAPPA_MIN && kap < KAPPA_MAX) ? 1.0 / (1.0 + exp(-pre)) : 0.0;
        m->logw[k] = o[5 * k + 4] - lz;
    }
}

static double logc(double k) { return log(k) - log(2.0 * M_PI) - k - log1p(-exp(-2.0 * k)); }

static double dlogc(double k)
{
    if (k < 1e-4) return -k / 3.0;
    return 1.0 / k - 1.0 / tanh(k);
}

static double mix_logpdf(const mix_t *m, const double *s, double *t)
{
    double tmax = -1e300;
    for (int k = 0; k < LP_COMP; ++k) {
        t[k] = m->logw[k] + logc(m->kappa[k]) + m->kappa[k] * (m->mu[k][0] * s[0] + m->mu[k][1] * s[1] + m->mu[k][2] * s[2]);
        tmax = fmax(tmax, t[k]);
    }
    double a = 0.0;
    for (int k = 0; k < LP_COMP; ++k) a += exp(t[k] - tmax);
    return tmax + log(a);
}

/* log q(s) of the mixture given by outputs o and kappa0, s a unit vector. */
double or_vmf_logpdf(const double *o, double kappa0, const double *s)
{
    mix_t m;
    double t[LP_COMP];
    mix_params(o, kappa0, &m);
    return mix_logpdf(&m, s, t);
}

/* A draw from the mixture with uniforms u[0..2] (component, cosine, azimuth). */
void or_vmf_sample(const double *o, double kappa0, const double *u, double *s)
{
    mix_t m;
    mix_params(o, kappa0, &m);
    int k = LP_COMP - 1;
    double c = 0.0;
    for (int j = 0; j < LP_COMP - 1; ++j) {
        c += exp(m.logw[j]);
        if (u[0] < c) { k = j; break; }
    }
    const double kap = m.kappa[k];
    double t = 1.0 + log1p((1.0 - u[1]) * expm1(-2.0 * kap)) / kap;
    t = fmin(fmax(t, -1.0), 1.0);
    const double r = sqrt(fmax(0.0, 1.0 - t * t));
    const double *mu = m.mu[k];
    double a[3] = {1.0, 0.0, 0.0};
    if (fabs(mu[0]) > 0.9) { a[0] = 0.0; a[1] = 1.0; }
    double e1[3] = {a[1] * mu[2] - a[2] * mu[1], a[2] * mu[0] - a[0] * mu[2], a[0] * mu[1] - a[1] * mu[0]};
    const double n1 = sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
    for (int i = 0; i < 3; ++i) e1[i] /= n1;
    const double e2[3] = {mu[1] * e1[2] - mu[2] * e1[1], mu[2] * e1[0] - mu[0] * e1[2], mu[0] * e1[1] - mu[1] * e1[0]};
    const double ph = 2.0 * M_PI * u[2];
    for (int i = 0; i < 3; ++i) s[i] = t * mu[i] + r * (cos(ph) * e1[i] + sin(ph) * e2[i]);
}

/* Mean negative log-likelihood of n samples and its gradient (LP_NPARAM
 * doubles).  x: (n,12) features; t: (n,4) unit spin in the local frame and
 * kappa0. */
double or_lp_loss_grad(const double *params, const double *x, const double *t, int64_t n, double *grad)
{
    lp_net net = net_of(params);
    memset(grad, 0, sizeof(double) * LP_NPARAM);
    lp_grad g = grad_of(grad);
    double h1[LP_HID], h2[LP_HID], o[LP_OUT], d_o[LP_OUT], dh2[LP_HID], dh1[LP_HID];
    double loss = 0.0;
    const double sc = 1.0 / (double)n;
    for (int64_t i = 0; i < n; ++i) {
        const double *xi = x + i * LP_IN, *ti = t + i * 4;
        forward1(&net, xi, h1, h2, o);
        mix_t m;
        double tk[LP_COMP];
        mix_params(o, ti[3], &m);
        const double lq = mix_logpdf(&m, ti, tk);
        loss -= lq * sc;
        for (int k = 0; k < LP_COMP; ++k) {
            const double r = exp(tk[k] - lq), w = exp(m.logw[k]);
            const double c = m.mu[k][0] * ti[0] + m.mu[k][1] * ti[1] + m.mu[k][2] * ti[2];
            const double gv = r * m.kappa[k] / m.vn[k];
            for (int a = 0; a < 3; ++a) d_o[5 * k + a] = -sc * gv * (ti[a] - c * m.mu[k][a]);
            d_o[5 * k + 3] = -sc * r * (dlogc(m.kappa[k]) + c) * m.dkappa[k];
            d_o[5 * k + 4] = -sc * (r - w);
        }
        for (int j = 0; j < LP_OUT; ++j) {
            g.b3[j] += d_o[j];
            for (int k = 0; k < LP_HID; ++k) g.w3[j * LP_HID + k] += d_o[j] * h2[k];
        }
        for (int k = 0; k < LP_HID; ++k) {
            double a = 0.0;
            for (int j = 0; j < LP_OUT; ++j) a += net.w3[j * LP_HID + k] * d_o[j];
            dh2[k] = h2[k] > 0.0 ? a : 0.0;
        }
        for (int j = 0; j < LP_HID; ++j) {
            g.b2[j] += dh2[j];
            for (int k = 0; k < LP_HID; ++k) g.w2[j * LP_HID + k] += dh2[j] * h1[k];
        }
        for (int k = 0; k < LP_HID; ++k) {
            double a = 0.0;
            for (int j = 0; j < LP_HID; ++j) a += net.w2[j * LP_HID + k] * dh2[j];
            dh1[k] = h1[k] > 0.0 ? a : 0.0;
        }
        for (int j = 0; j < LP_HID; ++j) {
            g.b1[j] += dh1[j];
            for (int k = 0; k < LP_IN; ++k) g.w1[j * LP_IN + k] += dh1[j] * xi[k];
        }
    }
    return loss;
}

/* Local frame and features of a site, as the sweep kernel computes them in
 * FP32 (lp_frame_features): frame rows e (9 doubles), kappa0, features f[12]. */
void or_lp_features(double beta, double mag, const double *g, const double *q, const double *axis, double *e,
                    double *kappa0, double *f)
{
    const double gn = sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
    const double k0 = beta * mag * gn;
    double e3[3] = {0.0, 0.0, 1.0};
    if (k0 > 1e-6) for (int i = 0; i < 3; ++i) e3[i] = -g[i] / gn;
    double d = axis[0] * e3[0] + axis[1] * e3[1] + axis[2] * e3[2];
    double e1[3] = {axis[0] - d * e3[0], axis[1] - d * e3[1], axis[2] - d * e3[2]};
    double n1 = e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2];
    if (n1 < 1e-6) {
        const double bx = fabs(e3[0]) < 0.9 ? 1.0 : 0.0, by = 1.0 - bx;
        d = bx * e3[0] + by * e3[1];
        e1[0] = bx - d * e3[0]; e1[1] = by - d * e3[1]; e1[2] = -d * e3[2];
        n1 = e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2];
    }
    n1 = sqrt(n1);
    for (int i = 0; i < 3; ++i) e1[i] /= n1;
    const double e2[3] = {e3[1] * e1[2] - e3[2] * e1[1], e3[2] * e1[0] - e3[0] * e1[2], e3[0] * e1[1] - e3[1] * e1[0]};
    const double *ev[3] = {e1, e2, e3};
    for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c) e[3 * a + c] = ev[a][c];
    const double Q[3][3] = {{q[0], q[3], q[4]}, {q[3], q[1], q[5]}, {q[4], q[5], q[2]}};
    double L[3][3];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            double v = 0.0;
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) v += ev[a][i] * Q[i][j] * ev[b][j];
            L[a][b] = v;
        }
    const double sc = beta * mag * mag;
    f[0] = log1p(k0);
    f[1] = 0.05 * k0;
    f[2] = sc * L[0][0]; f[3] = sc * L[1][1]; f[4] = sc * L[2][2];
    f[5] = sc * L[0][1]; f[6] = sc * L[0][2]; f[7] = sc * L[1][2];
    f[8] = sc * (L[0][0] + L[1][1] + L[2][2]);
    f[9] = sc * (L[2][2] - 0.5 * (L[0][0] + L[1][1]));
    f[10] = log(beta);
    f[11] = 1.0 / (1.0 + k0);
    *kappa0 = k0;
}
