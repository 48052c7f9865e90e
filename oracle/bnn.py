"""Bayesian neural network regression under KLqp (analytic KL).
Test infrastructure: see ``oracle/__init__.py``.

Model of ``examples/bayesian_nn.py:120-162`` with the layer sizes of the
benchmark configuration: h1 = tanh(X W0 + b0), h2 = tanh(h1 W1 + b1),
out = h2 W2 + b2, y ~ Normal(out, noise); every weight ~ Normal(0, 1);
q = mean-field Normal(mu, softplus(rho)).  The ELBO gradient is the one of
``build_reparam_kl_loss_and_gradients`` (``edward/inferences/klqp.py:707-769``)
with the minibatch scale N/M on the log-likelihood (``scale`` dict,
``edward/inferences/inference.py:215-220``).

Parameters are flattened in the order W0, b0, W1, b1, W2, b2 (row-major).
"""
import numpy as np

from . import densities as dn


def layer_sizes(D, H1, H2):
    return [(D, H1), (H1,), (H1, H2), (H2,), (H2, 1), (1,)]


def n_params(D, H1, H2):
    return sum(int(np.prod(s)) for s in layer_sizes(D, H1, H2))


def unpack(theta, D, H1, H2):
    out, o = [], 0
    for s in layer_sizes(D, H1, H2):
        n = int(np.prod(s))
        out.append(theta[..., o:o + n].reshape(theta.shape[:-1] + s))
        o += n
    return out


def forward(theta, X, D, H1, H2):
    """theta [S, P] -> (h1, h2, out) with out [S, M]."""
    W0, b0, W1, b1, W2, b2 = unpack(theta, D, H1, H2)
    h1 = np.tanh(np.einsum("md,sdh->smh", X, W0) + b0[:, None, :])
    h2 = np.tanh(np.einsum("smh,shk->smk", h1, W1) + b1[:, None, :])
    out = np.einsum("smk,sko->smo", h2, W2)[..., 0] + b2[:, None, 0]
    return h1, h2, out


def log_lik_and_grad(theta, X, y, noise, scale, D, H1, H2):
    """Per-sample scaled Gaussian log-likelihood [S] and its gradient [S, P]."""
    theta = np.asarray(theta, np.float64)
    X = np.asarray(X, np.float64)
    y = np.asarray(y, np.float64)
    W0, b0, W1, b1, W2, b2 = unpack(theta, D, H1, H2)
    h1, h2, out = forward(theta, X, D, H1, H2)
    res = y[None, :] - out                                      # [S, M]
    ll = scale * (-0.5 * (res / noise) ** 2 - np.log(noise) - dn.HALF_LOG_2PI).sum(axis=1)
    dout = scale * res / noise ** 2                             # d ll / d out
    gW2 = np.einsum("smk,sm->sk", h2, dout)[..., None]
    gb2 = dout.sum(axis=1)[:, None]
    dh2 = dout[..., None] * W2[:, None, :, 0] * (1.0 - h2 * h2)  # [S, M, H2]
    gW1 = np.einsum("smh,smk->shk", h1, dh2)
    gb1 = dh2.sum(axis=1)
    dh1 = np.einsum("smk,shk->smh", dh2, W1) * (1.0 - h1 * h1)
    gW0 = np.einsum("md,smh->sdh", X, dh1)
    gb0 = dh1.sum(axis=1)
    S = theta.shape[0]
    g = np.concatenate([a.reshape(S, -1) for a in (gW0, gb0, gW1, gb1, gW2, gb2)], axis=1)
    return ll, g


def klqp_loss_and_grads(mu, rho, eps, X, y, noise, scale, D, H1, H2, prior_scale=1.0,
                        method=0):
    """-ELBO and its gradient w.r.t. (mu, rho).  ``method`` 0: analytic KL to
    N(0, prior_scale) (``klqp.py:707-769``); 1: Monte Carlo KL,
    -mean_s[log p(x|z_s) + log p(z_s) - log q(z_s)] with the gradient through
    z_s and q's parameters (``klqp.py:642-704``)."""
    mu = np.asarray(mu, np.float64)
    rho = np.asarray(rho, np.float64)
    eps = np.asarray(eps, np.float64)
    sig = dn.softplus(rho)
    theta = mu[None, :] + sig[None, :] * eps
    ll, g = log_lik_and_grad(theta, X, y, noise, scale, D, H1, H2)
    if method == 0:
        kl = dn.kl_normal_normal(mu, sig, 0.0, prior_scale)
        dkl_mu, dkl_sig = dn.kl_normal_normal_grads(mu, sig, 0.0, prior_scale)
        loss = -(ll.mean() - kl.sum())
        gmu = -g.mean(axis=0) + dkl_mu
        gsig = -(g * eps).mean(axis=0) + dkl_sig
    else:
        lp = dn.normal_log_prob(theta, 0.0, prior_scale).sum(axis=1)
        lq = dn.normal_log_prob(theta, mu, sig).sum(axis=1)
        loss = -(ll + lp - lq).mean()
        dfdz = g - theta / prior_scale ** 2             # log q's z- and mu-terms cancel
        gmu = -dfdz.mean(axis=0)
        gsig = -(dfdz * eps).mean(axis=0) - 1.0 / sig
    return float(loss), gmu, gsig * dn.sigmoid(rho)


def synthetic(N, D, H1, H2, noise=0.1, seed=0):
    """X ~ N(0,1) [N, D]; y = random tanh net (weights N(0,1)/sqrt(fan_in)) + N(0, noise^2)."""
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((N, D)).astype(np.float32)
    W0 = rng.standard_normal((D, H1)) / np.sqrt(D)
    W1 = rng.standard_normal((H1, H2)) / np.sqrt(H1)
    W2 = rng.standard_normal((H2, 1)) / np.sqrt(H2)
    y = np.tanh(np.tanh(X @ W0) @ W1) @ W2
    y = (y[:, 0] + noise * rng.standard_normal(N)).astype(np.float32)
    return X, y


def minibatch_rows(seed, iteration, M, N):
    """Rows drawn by the device minibatch gather at one iteration: the first
    word of Philox stream 4, counter (0, m, iteration, 4), mapped to [0, N) by
    (u * N) >> 32."""
    from .philox import KIND_MINIBATCH, raw_u32
    u = raw_u32(seed, KIND_MINIBATCH, iteration, M, 1)[:, 0].astype(np.uint64)
    return ((u * np.uint64(N)) >> np.uint64(32)).astype(np.int64)

