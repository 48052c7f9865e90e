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

BLAS threads are whatever NumPy's BLAS is configured with (the caller sets
them to the number of host cores).
"""
import numpy as np

from .philox import KIND_EPS, KIND_MOMENTUM, KIND_UNIFORM, normals, uniforms64


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
