"""Generalised linear model family: y_n ~ Lik(eta_n), eta = X w (+ b),
Normal priors on every coordinate of z = (w, b).

Test infrastructure: see ``oracle/__init__.py``.

This is the model of ``examples/bayesian_logistic_regression.py`` /
``tests/inferences/hmc_test.py:48-91`` (``y = Normal(ed.dot(X, w) + b, 0.1)``)
and of the Normal-Normal tests (``klqp_test.py:14-44``: ``x = Normal(mu, 1)``,
i.e. X = ones(N, 1), no bias).  The contraction is ``ed.dot``
(``edward/util/tensorflow.py:41-47``: tf.matmul(X, expand_dims(w, 1))).

Log-likelihood terms are multiplied by ``data_scale`` (the ``scale`` dict of
``Inference.initialize``, ``edward/inferences/inference.py:215-220``; applied
by the KLqp builders at ``klqp.py:686,747`` and NOT by HMC, ``hmc.py:161-192``).
"""
from dataclasses import dataclass, field

import numpy as np

from . import densities as dn

BERNOULLI = 0
NORMAL = 1


@dataclass
class GLM:
    X: np.ndarray                 # [N, D]
    y: np.ndarray                 # [N]
    bias: bool = True
    lik: int = BERNOULLI
    lik_scale: float = 1.0        # Normal likelihood scale
    prior_loc: np.ndarray = None  # [P]
    prior_scale: np.ndarray = None
    data_scale: float = 1.0

    def __post_init__(self):
        self.X = np.asarray(self.X, np.float64)
        self.y = np.asarray(self.y, np.float64)
        P = self.P
        if self.prior_loc is None:
            self.prior_loc = np.zeros(P)
        if self.prior_scale is None:
            self.prior_scale = np.ones(P)
        self.prior_loc = np.broadcast_to(np.asarray(self.prior_loc, np.float64), (P,)).copy()
        self.prior_scale = np.broadcast_to(np.asarray(self.prior_scale, np.float64), (P,)).copy()

    @property
    def N(self):
        return self.X.shape[0]

    @property
    def D(self):
        return self.X.shape[1]

    @property
    def P(self):
        return self.D + (1 if self.bias else 0)

    def eta(self, Z, dtype=np.float64):
        """Linear predictor [N, B] for parameter vectors Z [B, P]."""
        Z = np.asarray(Z, dtype)
        X = self.X.astype(dtype)
        e = X @ Z[:, :self.D].T
        if self.bias:
            e = e + Z[:, self.D][None, :]
        return e

    def _terms(self, e):
        y = self.y.astype(e.dtype)[:, None]
        if self.lik == BERNOULLI:
            return dn.bernoulli_logits_log_prob(y, e), dn.bernoulli_logits_grad_logits(y, e)
        s = e.dtype.type(self.lik_scale)
        return dn.normal_log_prob(y, e, s), (y - e) / (s * s)

    def log_lik(self, Z, scaled=True, dtype=np.float64):
        """Sum over rows of the likelihood log density, per vector: [B]."""
        lp, _ = self._terms(self.eta(Z, dtype))
        out = lp.sum(axis=0, dtype=np.float64)
        return out * (self.data_scale if scaled else 1.0)

    def grad_log_lik(self, Z, scaled=True, dtype=np.float64):
        """Gradient of log_lik w.r.t. z: [B, P] (the adjoint X^T r)."""
        e = self.eta(Z, dtype)
        _, r = self._terms(e)
        X = self.X.astype(dtype)
        g = r.T @ X
        if self.bias:
            g = np.concatenate([g, r.sum(axis=0)[:, None]], axis=1)
        return g * (self.data_scale if scaled else 1.0)

    def log_prior(self, Z):
        Z = np.asarray(Z, np.float64)
        return dn.normal_log_prob(Z, self.prior_loc, self.prior_scale).sum(axis=1)

    def grad_log_prior(self, Z):
        Z = np.asarray(Z, np.float64)
        return dn.normal_grad_x(Z, self.prior_loc, self.prior_scale)

    def log_joint(self, Z, dtype=np.float64):
        """Unscaled prior + likelihood (the HMC target, ``hmc.py:161-192``)."""
        return self.log_prior(Z) + self.log_lik(Z, scaled=False, dtype=dtype)

    def grad_log_joint(self, Z, dtype=np.float64):
        return self.grad_log_prior(Z) + self.grad_log_lik(Z, scaled=False, dtype=dtype)


def synthetic_logreg(N, D, seed=0, dtype=np.float32):
    """The logistic-regression workload: X ~ N(0,1) [N, D], w* ~ N(0,1)^D,
    b* ~ N(0,1), y ~ Bernoulli(sigmoid(X w* + b*)).  Returns (X, y, w*, b*)."""
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((N, D)).astype(dtype)
    w = rng.standard_normal(D)
    b = rng.standard_normal()
    p = dn.sigmoid(X.astype(np.float64) @ w + b)
    y = (rng.random(N) < p).astype(dtype)
    return X, y, w, b


def conjugate_linreg_posterior(X, y, noise_std, prior_scale=1.0, bias=True):
    """Closed-form posterior N(m, S) of Bayesian linear regression
    y ~ N(X w + b, noise^2), w, b ~ N(0, prior_scale^2): the conjugate case
    behind ``tests/inferences/hmc_test.py:48-91``."""
    X = np.asarray(X, np.float64)
    if bias:
        X = np.concatenate([X, np.ones((X.shape[0], 1))], axis=1)
    prec = X.T @ X / noise_std ** 2 + np.eye(X.shape[1]) / prior_scale ** 2
    cov = np.linalg.inv(prec)
    mean = cov @ (X.T @ np.asarray(y, np.float64)) / noise_std ** 2
    return mean, cov
