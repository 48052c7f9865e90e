"""CPU restatement of the reference's hot path, structured the way the
reference executes it, used as the timed CPU baseline (``bench.py --impl
reference`` and the ``cpu_baseline`` field).  Test / benchmark
infrastructure: see ``oracle/__init__.py``.

TensorFlow 1.x (the reference's runtime) cannot be installed here, so this
module reproduces the reference's execution structure in NumPy FP32:

* HMC (``edward/inferences/hmc.py:61-130,195-210``): ONE chain per
  inference (the reference has no chain batching); each leapfrog step is a
  fresh log-joint graph: a GEMV over X (``ed.dot``,
  ``edward/util/tensorflow.py:41-47``), the Bernoulli log-prob, and a
  transposed GEMV for ``tf.gradients``; the Metropolis ratio adds two more
  log-joint evaluations without gradients (``hmc.py:100-105``): per
  iteration n_steps + 1 gradients and 2 plain log joints.
* KLqp (``klqp.py:707-769``): one model copy per Monte Carlo sample (GEMV
  forward + GEMV backward each), the analytic KL, then an unfused Adam apply
  (``variational_inference.py:97,120-121``).
* SGLD (``sgld.py:63-88``): one log-joint gradient graph per iteration (two
  GEMVs), the Langevin update with the Philox stream-5 noise.
* MetropolisHastings (``metropolis_hastings.py:64-156``): per iteration the
  proposal and two log-joint graphs, of the proposal and of the current
  state (one GEMV each), then the ratio and the test.
* HMC on one hierarchical instance (``hmc.py`` with the softplus transform
  of ``util/random_variables.py:903-904``): as the HMC chain above, with the
  Normal(mu, tau) prior of w, the priors of mu and tau and the log-det
  Jacobian added to every log joint and gradient.

BLAS threads are whatever NumPy's BLAS is configured with (the caller sets
them to the number of host cores).
"""
import numpy as np

from .philox import KIND_EPS, KIND_MOMENTUM, KIND_UNIFORM, normals, uniforms64

KIND_SGMCMC, KIND_MH_PROPOSAL, KIND_MH_UNIFORM = 5, 6, 7


def _softplus(x):
    return np.maximum(x, 0) + np.log1p(np.exp(-np.abs(x)))


def _sigmoid(x):
    return 0.5 * (1.0 + np.tanh(0.5 * x))


def _log_joint(X, y, w, b, prior_loc, prior_scale):
    """One reference log-joint graph without its gradient (one GEMV over X):
    the two Metropolis log joints of ``hmc.py:103-104``."""
    eta = X @ w + b                                              # ed.dot
    ll = -(np.maximum(eta, 0) - eta * y + np.log1p(np.exp(-np.abs(eta)))).sum(dtype=np.float32)
    z = np.concatenate([w, [b]]).astype(np.float32)
    zz = (z - prior_loc) / prior_scale
    lp = (-0.5 * zz * zz - np.log(prior_scale) - np.float32(0.9189385)).sum(dtype=np.float32)
    return np.float32(ll + lp)


def _log_joint_and_grad(X, y, w, b, prior_loc, prior_scale):
    """One reference log-joint graph + its gradient (two GEMVs over X)."""
    eta = X @ w + b                                              # ed.dot
    ll = -(np.maximum(eta, 0) - eta * y + np.log1p(np.exp(-np.abs(eta)))).sum(dtype=np.float32)
    z = np.concatenate([w, [b]]).astype(np.float32)
    zz = (z - prior_loc) / prior_scale
    lp = (-0.5 * zz * zz - np.log(prior_scale) - np.float32(0.9189385)).sum(dtype=np.float32)
    r = y - _sigmoid(eta)
    gw = X.T @ r                                                  # tf.gradients
    gb = r.sum(dtype=np.float32)
    g = np.concatenate([gw, [gb]]).astype(np.float32) - (z - prior_loc) / prior_scale ** 2
    return np.float32(ll + lp), g.astype(np.float32)


def hmc_logreg_chain(X, y, z0, n_iter, step_size, n_steps, seed, chain, prior_loc, prior_scale):
    """n_iter reference-structured HMC iterations of one chain; returns
    (final state, n_accept)."""
    X = np.asarray(X, np.float32)
    y = np.asarray(y, np.float32)
    D = X.shape[1]
    z = np.asarray(z0, np.float32).copy()
    eps = np.float32(step_size)
    n_acc = 0
    for t in range(n_iter):
        r0 = normals(seed, KIND_MOMENTUM, t, 1, D + 1, row0=chain)[0].astype(np.float32)
        u = uniforms64(seed, KIND_UNIFORM, t, 1, row0=chain)[0]
        zn, r = z.copy(), r0.copy()
        _, g = _log_joint_and_grad(X, y, zn[:D], zn[D], prior_loc, prior_scale)
        for _ in range(n_steps):
            r = r + np.float32(0.5) * eps * g
            zn = zn + eps * r
            _, g = _log_joint_and_grad(X, y, zn[:D], zn[D], prior_loc, prior_scale)
            r = r + np.float32(0.5) * eps * g
        lj_new = _log_joint(X, y, zn[:D], zn[D], prior_loc, prior_scale)
        lj_old = _log_joint(X, y, z[:D], z[D], prior_loc, prior_scale)
        ratio = 0.5 * (r0 * r0).sum() - 0.5 * (r * r).sum() + lj_new - lj_old
        if np.log(u) < ratio:
            z = zn
            n_acc += 1
    return z, n_acc


def sgld_logreg_chain(X, y, z0, n_iter, step_size, seed, chain, prior_loc, prior_scale):
    """n_iter reference-structured SGLD iterations of one chain (full data,
    scale 1); returns the final state."""
    X = np.asarray(X, np.float32)
    y = np.asarray(y, np.float32)
    D = X.shape[1]
    z = np.asarray(z0, np.float32).copy()
    for t in range(n_iter):
        _, g = _log_joint_and_grad(X, y, z[:D], z[D], prior_loc, prior_scale)
        e = normals(seed, KIND_SGMCMC, t, 1, D + 1, row0=chain)[0].astype(np.float32)
        lr = np.float32(step_size / (t + 1.0) ** 0.55)
        z = z + np.float32(0.5) * lr * g + np.sqrt(lr) * e
    return z


def mh_logreg_chain(X, y, z0, n_iter, scale, seed, chain, prior_loc, prior_scale):
    """n_iter reference-structured random-walk Metropolis-Hastings iterations
    of one chain; returns (final state, n_accept)."""
    X = np.asarray(X, np.float32)
    y = np.asarray(y, np.float32)
    D = X.shape[1]
    z = np.asarray(z0, np.float32).copy()
    n_acc = 0
    for t in range(n_iter):
        e = normals(seed, KIND_MH_PROPOSAL, t, 1, D + 1, row0=chain)[0].astype(np.float32)
        zn = z + np.asarray(scale, np.float32) * e
        lj_new = _log_joint(X, y, zn[:D], zn[D], prior_loc, prior_scale)
        lj_old = _log_joint(X, y, z[:D], z[D], prior_loc, prior_scale)
        u = uniforms64(seed, KIND_MH_UNIFORM, t, 1, row0=chain)[0]
        if np.log(u) < float(lj_new) - float(lj_old):
            z = zn
            n_acc += 1
    return z, n_acc


def _hier_log_joint(X, y, w, mu, u, mu_loc, mu_scale, tau_scale, grad):
    """One hierarchical log-joint graph (one GEMV over X_i, plus its
    transposed GEMV with ``grad``): Bernoulli likelihood, w ~ N(mu, tau),
    mu ~ N(mu_loc, mu_scale), tau ~ HalfNormal(tau_scale) with tau =
    softplus(u) and log|d tau / d u| = log sigmoid(u)."""
    eta = X @ w                                                   # ed.dot
    ll = -(np.maximum(eta, 0) - eta * y + np.log1p(np.exp(-np.abs(eta)))).sum(dtype=np.float32)
    tau = np.float32(_softplus(u))
    dev = w - mu
    D = w.shape[0]
    s2 = np.float32((dev * dev).sum(dtype=np.float32))
    lw = -0.5 * s2 / (tau * tau) - D * np.log(tau) - D * np.float32(0.9189385)
    zm = (mu - mu_loc) / mu_scale
    lmu = -0.5 * zm * zm - np.log(mu_scale) - np.float32(0.9189385)
    zt = tau / tau_scale
    ltau = np.float32(0.5 * np.log(2.0 / np.pi)) - np.log(tau_scale) - 0.5 * zt * zt
    ldj = -_softplus(-u)
    lj = np.float32(ll + lw + lmu + ltau + ldj)
    if not grad:
        return lj, None
    r = y - _sigmoid(eta)
    gw = (X.T @ r - dev / (tau * tau)).astype(np.float32)         # tf.gradients
    gmu = np.float32(dev.sum(dtype=np.float32) / (tau * tau) - (mu - mu_loc) / mu_scale ** 2)
    dtau = -D / tau + s2 / tau ** 3 - tau / tau_scale ** 2
    sg = np.float32(_sigmoid(u))
    gu = np.float32(dtau * sg + (1.0 - sg))
    return lj, np.concatenate([gw, [gmu, gu]]).astype(np.float32)


def hier_chain(X, y, z0, n_iter, step_size, n_steps, seed, chain, mu_loc=0.0, mu_scale=1.0,
               tau_scale=1.0):
    """n_iter reference-structured HMC iterations of one chain of one
    hierarchical instance, state (w [D], mu, u); returns (final state,
    n_accept).  Momenta and uniforms use Philox streams 1 and 2 at global
    chain row ``chain``, as the kernels do."""
    X = np.asarray(X, np.float32)
    y = np.asarray(y, np.float32)
    D = X.shape[1]
    z = np.asarray(z0, np.float32).copy()
    eps = np.float32(step_size)
    args = (np.float32(mu_loc), np.float32(mu_scale), np.float32(tau_scale))
    n_acc = 0
    for t in range(n_iter):
        r0 = normals(seed, KIND_MOMENTUM, t, 1, D + 2, row0=chain)[0].astype(np.float32)
        u = uniforms64(seed, KIND_UNIFORM, t, 1, row0=chain)[0]
        zn, r = z.copy(), r0.copy()
        _, g = _hier_log_joint(X, y, zn[:D], zn[D], zn[D + 1], *args, True)
        for _ in range(n_steps):
            r = r + np.float32(0.5) * eps * g
            zn = zn + eps * r
            _, g = _hier_log_joint(X, y, zn[:D], zn[D], zn[D + 1], *args, True)
            r = r + np.float32(0.5) * eps * g
        lj_new, _ = _hier_log_joint(X, y, zn[:D], zn[D], zn[D + 1], *args, False)
        lj_old, _ = _hier_log_joint(X, y, z[:D], z[D], z[D + 1], *args, False)
        ratio = 0.5 * (r0 * r0).sum() - 0.5 * (r * r).sum() + lj_new - lj_old
        if np.log(u) < ratio:
            z = zn
            n_acc += 1
    return z, n_acc


def klqp_logreg_step(X, y, mu, rho, m, v, t, n_samples, seed, prior_loc, prior_scale, lr):
    """One reference-structured KLqp (analytic KL) step with TF Adam; updates
    mu, rho, m, v in place and returns the loss."""
    X = np.asarray(X, np.float32)
    y = np.asarray(y, np.float32)
    D = X.shape[1]
    P = D + 1
    sig = _softplus(rho).astype(np.float32)
    eps = normals(seed, KIND_EPS, t, n_samples, P).astype(np.float32)
    gmu = np.zeros(P, np.float32)
    gsig = np.zeros(P, np.float32)
    ll_sum = np.float32(0.0)
    for s in range(n_samples):                     # one model copy per sample
        z = mu + sig * eps[s]
        eta = X @ z[:D] + z[D]
        ll_sum += -(np.maximum(eta, 0) - eta * y + np.log1p(np.exp(-np.abs(eta)))).sum(dtype=np.float32)
        r = y - _sigmoid(eta)
        g = np.concatenate([X.T @ r, [r.sum()]]).astype(np.float32)
        gmu -= g / n_samples
        gsig -= g * eps[s] / n_samples
    ratio = (sig / prior_scale) ** 2
    kl = (0.5 * ((mu - prior_loc) / prior_scale) ** 2 + 0.5 * (ratio - 1 - np.log(ratio))).sum()
    gmu += (mu - prior_loc) / prior_scale ** 2
    gsig += sig / prior_scale ** 2 - 1.0 / sig
    grho = gsig * _sigmoid(rho)
    loss = -(ll_sum / n_samples - kl)
    g = np.concatenate([gmu, grho])
    theta = np.concatenate([mu, rho])
    b1, b2 = 0.9, 0.999
    lr_t = lr * np.sqrt(1 - b2 ** (t + 1)) / (1 - b1 ** (t + 1))
    m[:] = b1 * m + (1 - b1) * g
    v[:] = b2 * v + (1 - b2) * g * g
    theta = theta - lr_t * m / (np.sqrt(v) + 1e-8)
    mu[:] = theta[:P]
    rho[:] = theta[P:]
    return float(loss)


def _adam(theta, g, m, v, t, lr):
    b1, b2 = 0.9, 0.999
    lr_t = lr * np.sqrt(1 - b2 ** (t + 1)) / (1 - b1 ** (t + 1))
    m[:] = b1 * m + (1 - b1) * g
    v[:] = b2 * v + (1 - b2) * g * g
    return theta - lr_t * m / (np.sqrt(v) + 1e-8)


def bnn_klqp_step(X, y, mu, rho, m, v, t, n_samples, seed, noise, scale, D, H1, H2, lr):
    """One reference-structured Bayesian-NN KLqp step (analytic KL,
    ``klqp.py:707-769`` on ``examples/bayesian_nn.py:120-162``): one copy of
    the network per Monte Carlo sample (three matmuls forward and their
    transposes for ``tf.gradients``), the analytic KL and an unfused Adam;
    NumPy FP32.  Updates mu, rho, m, v in place and returns the loss."""
    X = np.asarray(X, np.float32)
    y = np.asarray(y, np.float32)
    P = mu.shape[0]
    sig = _softplus(rho).astype(np.float32)
    eps = normals(seed, KIND_EPS, t, n_samples, P).astype(np.float32)
    gmu = np.zeros(P, np.float32)
    gsig = np.zeros(P, np.float32)
    ll_sum = 0.0
    n0, n1, n2 = D * H1, H1 * H2, H2
    for s in range(n_samples):                     # one model copy per sample
        th = mu + sig * eps[s]
        W0 = th[:n0].reshape(D, H1)
        b0 = th[n0:n0 + H1]
        o = n0 + H1
        W1 = th[o:o + n1].reshape(H1, H2)
        b1 = th[o + n1:o + n1 + H2]
        o += n1 + H2
        W2 = th[o:o + n2].reshape(H2, 1)
        b2 = th[o + n2]
        h1 = np.tanh(X @ W0 + b0)
        h2 = np.tanh(h1 @ W1 + b1)
        res = y - (h2 @ W2)[:, 0] - b2
        ll_sum += float(scale * ((-0.5 * (res / noise) ** 2).sum(dtype=np.float32)
                                 - res.shape[0] * (np.log(noise) + 0.9189385332)))
        dout = (scale * res / noise ** 2).astype(np.float32)
        dh2 = np.outer(dout, W2[:, 0]) * (1.0 - h2 * h2)
        dh1 = (dh2 @ W1.T) * (1.0 - h1 * h1)
        g = np.concatenate([(X.T @ dh1).reshape(-1), dh1.sum(0), (h1.T @ dh2).reshape(-1),
                            dh2.sum(0), h2.T @ dout, [dout.sum()]]).astype(np.float32)
        gmu -= g / n_samples
        gsig -= g * eps[s] / n_samples
    kl = (0.5 * mu * mu + 0.5 * (sig * sig - 1.0) - np.log(sig)).sum()
    gmu += mu
    gsig += sig - 1.0 / sig
    grho = gsig * _sigmoid(rho)
    theta = _adam(np.concatenate([mu, rho]), np.concatenate([gmu, grho]), m, v, t, lr)
    mu[:] = theta[:P]
    rho[:] = theta[P:]
    return -(ll_sum / n_samples - kl)


def sbn_score_step(X, theta, m, v, t, n_samples, seed, V, H0, H1, lr):
    """One reference-structured ScoreKLqp step on the sigmoid belief network
    (``build_score_loss_and_gradients``, ``klqp.py:840-906``, model of
    ``examples/sigmoid_belief_network.py:54-86``): per Monte Carlo sample a
    copy of q (784 -> 200 -> 200, Bernoulli draws) and of p (200 -> 200 -> 784),
    the per-sample learning signal log p - log q, and the score and
    reparameterisation-free gradients through transposed matmuls; unfused
    Adam; NumPy FP32.  Updates theta, m, v in place and returns the loss."""
    X = np.asarray(X, np.float32)
    B = X.shape[0]
    rng = np.random.default_rng(seed * 1000003 + t)
    shapes = [(V + 1, H0), (H0 + 1, H1), (H1 + 1, H0), (H0 + 1, V)]
    Ws, o = [], 0
    for r, c in shapes:
        Ws.append(theta[o:o + r * c].reshape(r, c))
        o += r * c
    Wq0, Wq1, Wp1, Wp0 = Ws
    aug = lambda a: np.concatenate([a, np.ones((a.shape[0], 1), np.float32)], 1)  # noqa: E731
    blogp = lambda z, lg: (z * lg - _softplus(lg)).sum(-1)                           # noqa: E731
    Xa = aug(X)
    g = [np.zeros_like(W) for W in Ws]
    F_sum = 0.0
    for _ in range(n_samples):                     # one copy of q and p per sample
        Lq0 = Xa @ Wq0
        z0 = (rng.random(Lq0.shape, dtype=np.float32) < _sigmoid(Lq0)).astype(np.float32)
        Z0a = aug(z0)
        Lq1 = Z0a @ Wq1
        z1 = (rng.random(Lq1.shape, dtype=np.float32) < _sigmoid(Lq1)).astype(np.float32)
        Z1a = aug(z1)
        Lp1 = Z1a @ Wp1
        Lp0 = Z0a @ Wp0
        f = (blogp(z1, np.zeros_like(z1)) + blogp(z0, Lp1) + blogp(X, Lp0)
             - blogp(z0, Lq0) - blogp(z1, Lq1))
        F = float(f.sum())
        F_sum += F
        g[0] -= Xa.T @ (F * (z0 - _sigmoid(Lq0))) / n_samples
        g[1] -= Z0a.T @ (F * (z1 - _sigmoid(Lq1))) / n_samples
        g[2] -= Z1a.T @ (z0 - _sigmoid(Lp1)) / n_samples
        g[3] -= Z0a.T @ (X - _sigmoid(Lp0)) / n_samples
    grad = np.concatenate([a.reshape(-1) for a in g]).astype(np.float32)
    theta[:] = _adam(theta, grad, m, v, t, lr)
    return -F_sum / n_samples / B
