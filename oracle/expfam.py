"""One constrained latent with i.i.d. observations, sampled / fitted in the
unconstrained space that ``auto_transform`` maps it to (FP64).  Test
infrastructure: see ``oracle/__init__.py``.

Families (``edward/util/random_variables.py:856-917`` picks the bijector from
the latent's support; ``edward/inferences/inference.py:222-264`` applies it):

* BETA:      z ~ Beta(a, b)        (support '01'),        x_i ~ Bernoulli(probs=z);
             z = sigmoid(u),       log|dz/du| = log sigmoid(u) + log sigmoid(-u)
* GAMMA:     z ~ Gamma(a, rate b)  (support 'nonnegative'), x_i ~ Poisson(rate=z);
             z = softplus(u),      log|dz/du| = log sigmoid(u)
* DIRICHLET: z ~ Dirichlet(alpha)  (support 'simplex'),   x_i ~ Categorical(probs=z);
             z = softmax([u, 0]) (SoftmaxCentered, u in R^(K-1)),
             log|det dz/du| = sum_k log z_k

The observations enter through sufficient statistics ``stats``: BETA (n1, n0),
GAMMA (sum x, N, sum log x!), DIRICHLET (counts[K]).  ``log_joint(u)`` is the
target HMC samples and the ``log p`` of KLqp's reparameterisation gradient.
"""
import numpy as np
from scipy.special import gammaln

from . import densities as dn

BETA, GAMMA, DIRICHLET = 0, 1, 2


def constrain(family, U):
    U = np.asarray(U, np.float64)
    if family == BETA:
        return dn.sigmoid(U)
    if family == GAMMA:
        return dn.softplus(U)
    ext = np.concatenate([U, np.zeros(U.shape[:-1] + (1,))], axis=-1)
    ext = ext - ext.max(axis=-1, keepdims=True)
    e = np.exp(ext)
    return e / e.sum(axis=-1, keepdims=True)


def log_joint_support(family, prior, stats, Z):
    """log p(x, z) on the support itself (no bijector, ``auto_transform=False``;
    Beta and Gamma): NaN where z is outside the support, as the reference's
    densities give for such draws (``inference_auto_transform_test.py:46-63``)."""
    z = np.asarray(Z, np.float64)[..., 0]
    with np.errstate(invalid="ignore", divide="ignore"):
        if family == BETA:
            a, b = prior
            n1, n0 = stats
            inside = (z > 0) & (z < 1)
            lp = (a - 1 + n1) * np.log(z) + (b - 1 + n0) * np.log1p(-z) - \
                (gammaln(a) + gammaln(b) - gammaln(a + b))
        else:
            a, rate = prior
            sx, n, slf = stats
            inside = z > 0
            lp = a * np.log(rate) - gammaln(a) + (a - 1 + sx) * np.log(z) - (rate + n) * z - slf
    return np.where(inside, lp, np.nan)


def grad_log_joint_support(family, prior, stats, Z):
    """d log_joint_support / d z (NaN outside the support), same shape as Z."""
    Z = np.asarray(Z, np.float64)
    with np.errstate(invalid="ignore", divide="ignore"):
        if family == BETA:
            a, b = prior
            n1, n0 = stats
            g = (a - 1 + n1) / Z - (b - 1 + n0) / (1 - Z)
            inside = (Z > 0) & (Z < 1)
        else:
            a, rate = prior
            sx, n, _ = stats
            g = (a - 1 + sx) / Z - rate - n
            inside = Z > 0
    return np.where(inside, g, np.nan)


def log_joint(family, prior, stats, U):
    """log p(x, z(u)) + log|det dz/du| for U [..., K'] (K' = 1, or K - 1)."""
    U = np.asarray(U, np.float64)
    if family == BETA:
        a, b = prior
        n1, n0 = stats
        u = U[..., 0]
        lz, l1z = -dn.softplus(-u), -dn.softplus(u)           # log z, log (1 - z)
        lp = (a - 1) * lz + (b - 1) * l1z - (gammaln(a) + gammaln(b) - gammaln(a + b))
        return lp + n1 * lz + n0 * l1z + lz + l1z
    if family == GAMMA:
        a, rate = prior
        sx, n, slf = stats
        u = U[..., 0]
        z = dn.softplus(u)
        lz = np.log(z)
        lp = a * np.log(rate) - gammaln(a) + (a - 1) * lz - rate * z
        return lp + sx * lz - n * z - slf - dn.softplus(-u)
    alpha = np.asarray(prior, np.float64)
    counts = np.asarray(stats, np.float64)
    z = constrain(DIRICHLET, U)
    lz = np.log(z)
    lp = ((alpha - 1) * lz).sum(-1) + gammaln(alpha.sum()) - gammaln(alpha).sum()
    return lp + (counts * lz).sum(-1) + lz.sum(-1)


def grad_log_joint(family, prior, stats, U):
    """d log_joint / d u, same shape as U."""
    U = np.asarray(U, np.float64)
    if family == BETA:
        a, b = prior
        n1, n0 = stats
        s = dn.sigmoid(U)
        # d log z / du = 1 - s, d log(1 - z) / du = -s
        return (a + n1) * (1 - s) - (b + n0) * s
    if family == GAMMA:
        a, rate = prior
        sx, n, _ = stats
        z = dn.softplus(U)
        dz = dn.sigmoid(U)
        return ((a - 1 + sx) / z - rate - n) * dz + dn.sigmoid(-U)
    alpha = np.asarray(prior, np.float64)
    counts = np.asarray(stats, np.float64)
    z = constrain(DIRICHLET, U)
    w = alpha - 1 + counts + 1                                 # coefficient of log z_k
    # d/du_j sum_k w_k log z_k = w_j - z_j sum_k w_k  (j < K - 1)
    return w[:-1] - z[..., :-1] * w.sum()


def sufficient_stats(family, x, K=None):
    x = np.asarray(x)
    if family == BETA:
        n1 = float((x == 1).sum())
        return n1, float(x.size) - n1
    if family == GAMMA:
        return float(x.sum()), float(x.size), float(gammaln(x + 1.0).sum())
    return np.bincount(x.astype(np.int64).reshape(-1), minlength=K).astype(np.float64)


def klqp_loss_and_grads(family, prior, stats, mu, rho, eps, transform=True):
    """-ELBO of q(u) = N(mu, softplus(rho)) with Monte Carlo KL
    (``klqp.py:642-704``) and its gradient w.r.t. (mu, rho), for draws eps [S, K];
    transform=False: q is on the support itself (``log_joint_support``)."""
    mu = np.asarray(mu, np.float64)
    rho = np.asarray(rho, np.float64)
    eps = np.asarray(eps, np.float64)
    sig = dn.softplus(rho)
    U = mu[None] + sig[None] * eps
    lj = (log_joint if transform else log_joint_support)(family, prior, stats, U)
    lq = (-0.5 * eps ** 2 - np.log(sig)[None] - dn.HALF_LOG_2PI).sum(-1)
    g = (grad_log_joint if transform else grad_log_joint_support)(family, prior, stats, U)
    loss = -(lj - lq).mean()
    gmu = -g.mean(0)
    gsig = -(g * eps).mean(0) - 1.0 / sig
    return float(loss), gmu, gsig * dn.sigmoid(rho)
