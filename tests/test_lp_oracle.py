"""CPU checks of the learned proposal's FP64 restatement (oracle/lp_oracle.c):
the loss gradient against finite differences (and torch autograd in FP64), the
mixture density's normalisation on the sphere, the sampler against the
density's moments, and the rotation invariance of the site features."""
import numpy as np
import pytest

import oracle as O


def _params(seed, scale=0.2):
    rng = np.random.default_rng(seed)
    p = rng.normal(size=O.lp_num_params()) * scale
    return p


def _data(seed, n):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n, 12))
    s = rng.normal(size=(n, 3))
    s /= np.linalg.norm(s, axis=1, keepdims=True)
    k0 = np.abs(rng.normal(size=n)) * 4.0
    return x, np.column_stack([s, k0])


def test_gradient_matches_central_differences():
    p = _params(1)
    x, t = _data(2, 16)
    loss, g = O.lp_loss_grad(p, x, t)
    assert np.isfinite(loss)
    rng = np.random.default_rng(3)
    # one index in every parameter block plus random ones
    blocks = [0, 1536, 1664, 18048, 18176, 20736]
    idx = np.concatenate([np.array(blocks) + 3, rng.choice(p.size, 40, replace=False)])
    for i in idx:
        e = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[i] += e
        pm[i] -= e
        fd = (O.lp_loss_grad(pp, x, t)[0] - O.lp_loss_grad(pm, x, t)[0]) / (2 * e)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])


def test_gradient_matches_torch_autograd_fp64():
    torch = pytest.importorskip("torch")
    p = _params(4)
    x, t = _data(5, 32)
    loss, g = O.lp_loss_grad(p, x, t)
    P = torch.tensor(p, dtype=torch.float64, requires_grad=True)
    o = 0
    W1 = P[o:o + 1536].view(128, 12); o += 1536
    b1 = P[o:o + 128]; o += 128
    W2 = P[o:o + 16384].view(128, 128); o += 16384
    b2 = P[o:o + 128]; o += 128
    W3 = P[o:o + 2560].view(20, 128); o += 2560
    b3 = P[o:o + 20]
    X = torch.tensor(x)
    T = torch.tensor(t)
    out = torch.relu(torch.relu(X @ W1.T + b1) @ W2.T + b2) @ W3.T + b3
    out = out.view(-1, 4, 5)
    v = torch.stack([out[..., 0], out[..., 1], 1.0 + out[..., 2]], dim=-1)
    mu = v / v.norm(dim=-1, keepdim=True)
    k0 = T[:, 3:4].clamp(min=1e-4)
    k0i = torch.where(k0 > 20, k0 + torch.log1p(-torch.exp(-k0)), torch.log(torch.expm1(k0)))
    kap = torch.nn.functional.softplus(out[..., 3] + k0i).clamp(1e-3, 1e4)
    logw = torch.log_softmax(out[..., 4], dim=-1)
    logc = torch.log(kap) - np.log(2 * np.pi) - kap - torch.log1p(-torch.exp(-2 * kap))
    lt = logw + logc + kap * (mu * T[:, None, :3]).sum(-1)
    L = -torch.logsumexp(lt, dim=-1).mean()
    L.backward()
    assert abs(L.item() - loss) <= 1e-10 * max(1.0, abs(loss))
    assert np.max(np.abs(P.grad.numpy() - g)) <= 1e-10 * max(1.0, np.abs(g).max())


def _sphere_grid(nt=2000, nph=400):
    ct = -1 + (np.arange(nt) + 0.5) * (2.0 / nt)
    ph = (np.arange(nph) + 0.5) * (2 * np.pi / nph)
    st = np.sqrt(1 - ct ** 2)
    s = np.stack([np.outer(st, np.cos(ph)), np.outer(st, np.sin(ph)), np.outer(ct, np.ones(nph))], -1).reshape(-1, 3)
    return s, (2.0 / nt) * (2 * np.pi / nph)


@pytest.mark.parametrize("kappa0", [0.0, 0.5, 5.0, 40.0])
def test_mixture_density_is_normalised(kappa0):
    rng = np.random.default_rng(int(kappa0 * 10) + 7)
    o = rng.normal(size=20)
    o[3::5] = np.clip(o[3::5], -3, 3)
    s, dw = _sphere_grid()
    lq = np.array([O.vmf_logpdf(o, kappa0, v) for v in s[::1]])
    total = np.exp(lq).sum() * dw
    assert abs(total - 1.0) < 2e-3, total


def test_sampler_reproduces_the_density_moments():
    rng = np.random.default_rng(11)
    o = rng.normal(size=20)
    kappa0 = 3.0
    u = rng.random(size=(60000, 3))
    x = np.array([O.vmf_sample(o, kappa0, ui) for ui in u])
    assert np.allclose(np.linalg.norm(x, axis=1), 1.0, atol=1e-12)
    s, dw = _sphere_grid(1000, 300)
    q = np.exp([O.vmf_logpdf(o, kappa0, v) for v in s]) * dw
    m1 = (q[:, None] * s).sum(0)
    m2 = (q[:, None, None] * s[:, :, None] * s[:, None, :]).sum(0)
    se = 5.0 / np.sqrt(len(x))
    assert np.all(np.abs(x.mean(0) - m1) < se), (x.mean(0), m1)
    assert np.all(np.abs((x[:, :, None] * x[:, None, :]).mean(0) - m2) < se)


def _rot(rng):
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    return q * np.sign(np.linalg.det(q))


def test_features_are_rotation_invariant_and_frame_is_orthonormal():
    rng = np.random.default_rng(5)
    for _ in range(20):
        g = rng.normal(size=3) * 30
        A = rng.normal(size=(3, 3))
        Q = A + A.T
        axis = rng.normal(size=3)
        axis /= np.linalg.norm(axis)
        q6 = [Q[0, 0], Q[1, 1], Q[2, 2], Q[0, 1], Q[0, 2], Q[1, 2]]
        e, k0, f = O.lp_features(0.1, 1.3, g, q6, axis)
        assert np.allclose(e @ e.T, np.eye(3), atol=1e-12)
        assert np.allclose(e[2], -g / np.linalg.norm(g))
        assert abs(k0 - 0.1 * 1.3 * np.linalg.norm(g)) < 1e-12
        Rm = _rot(rng)
        Q2 = Rm @ Q @ Rm.T
        q62 = [Q2[0, 0], Q2[1, 1], Q2[2, 2], Q2[0, 1], Q2[0, 2], Q2[1, 2]]
        e2, k02, f2 = O.lp_features(0.1, 1.3, Rm @ g, q62, Rm @ axis)
        assert np.allclose(f, f2, atol=1e-9)
        assert np.allclose(e2, e @ Rm.T, atol=1e-9)


def test_zero_outputs_give_the_heisenberg_conditional():
    """With zero network outputs the mixture is vMF(e3, kappa0): the exact
    conditional of a site with only a linear field."""
    o = np.zeros(20)
    for k0 in (0.01, 1.0, 30.0):
        for c in (-0.9, 0.0, 0.7, 1.0):
            s = np.array([np.sqrt(1 - c * c), 0.0, c])
            want = np.log(k0 / (4 * np.pi * np.sinh(k0))) + k0 * c
            assert abs(O.vmf_logpdf(o, k0, s) - want) < 1e-9
