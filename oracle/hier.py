"""Hierarchical logistic regression, one model instance per (X_i, y_i).
Test infrastructure: see ``oracle/__init__.py``.

    mu ~ Normal(mu_loc, mu_scale),  tau ~ HalfNormal(tau_scale),
    w_d ~ Normal(mu, tau) for d < D,  y_n ~ Bernoulli(logits = X_n . w)

HMC runs on the unconstrained coordinates z = (w, mu, u) with tau = softplus(u):
``inference.initialize(auto_transform=True)`` maps a latent whose support is
'nonnegative' through ``Invert(Softplus())`` (``edward/util/random_variables.py:903-904``,
``edward/inferences/inference.py:224-264``) and ``_log_joint_unconstrained``
adds the inverse transform's log-det-Jacobian ``log sigmoid(u)``
(``edward/inferences/hmc.py:145-159``).  HalfNormal needs
``tau.support = 'nonnegative'`` set by the user (the reference tags no support
on it, ``edward/models/random_variables.py:29-43``).
"""
import numpy as np

from . import densities as dn


def log_joint_grad(X, y, Z, mu_loc=0.0, mu_scale=1.0, tau_scale=1.0):
    """(lj [C], grad [C, D+2]) for chain states Z [C, D+2] = (w, mu, u)."""
    X = np.asarray(X, np.float64)
    y = np.asarray(y, np.float64)
    Z = np.asarray(Z, np.float64)
    D = X.shape[1]
    w, mu, u = Z[:, :D], Z[:, D], Z[:, D + 1]
    tau = dn.softplus(u)
    eta = X @ w.T                                        # [N, C]
    ll = dn.bernoulli_logits_log_prob(y[:, None], eta).sum(axis=0)
    r = y[:, None] - dn.sigmoid(eta)
    dev = w - mu[:, None]
    s1 = dev.sum(axis=1)
    s2 = (dev * dev).sum(axis=1)
    lp_w = -0.5 * s2 / tau ** 2 - D * np.log(tau) - D * dn.HALF_LOG_2PI
    lp_mu = dn.normal_log_prob(mu, mu_loc, mu_scale)
    lp_tau = dn.half_normal_log_prob(tau, tau_scale)
    ldj = -dn.softplus(-u)                               # log sigmoid(u)
    lj = ll + lp_w + lp_mu + lp_tau + ldj
    gw = r.T @ X - dev / tau[:, None] ** 2
    gmu = s1 / tau ** 2 - (mu - mu_loc) / mu_scale ** 2
    dtau = -D / tau + s2 / tau ** 3 - tau / tau_scale ** 2
    sig = dn.sigmoid(u)
    gu = dtau * sig + (1.0 - sig)
    return lj, np.concatenate([gw, gmu[:, None], gu[:, None]], axis=1)


def lj_grad_fn(X, y, **kw):
    def f(Z):
        return log_joint_grad(X, y, Z, **kw)
    return f


def synthetic_instances(I, seed=0, n_range=(50, 20000), d_range=(8, 128), dtype=np.float32):
    """I ragged instances: N_i log-uniform in n_range, D_i uniform in d_range,
    X ~ N(0,1), w_i ~ N(mu_i, tau_i^2) with mu_i ~ N(0,1), tau_i ~ HalfNormal(1),
    y ~ Bernoulli(sigmoid(X w_i)).  Returns lists (Xs, ys)."""
    rng = np.random.default_rng(seed)
    Xs, ys = [], []
    lo, hi = np.log(n_range[0]), np.log(n_range[1])
    for _ in range(I):
        N = int(np.exp(rng.uniform(lo, hi)))
        D = int(rng.integers(d_range[0], d_range[1] + 1))
        X = rng.standard_normal((N, D)).astype(dtype)
        mu = rng.standard_normal()
        tau = abs(rng.standard_normal())
        w = mu + tau * rng.standard_normal(D)
        p = dn.sigmoid(X.astype(np.float64) @ w)
        y = (rng.random(N) < p).astype(dtype)
        Xs.append(X)
        ys.append(y)
    return Xs, ys
