"""KLqp ELBO gradients for a mean-field Normal q over a GLM, TF's Adam and the
default learning-rate schedule.  Test infrastructure: see ``oracle/__init__.py``.

q(z) = N(mu, softplus(rho)) elementwise, the default family that ``KLqp``
builds for list latents (``edward/inferences/klqp.py:76-80``) and that the
reference's own tests and examples build by hand
(``tests/inferences/klqp_test.py:22-24``).

Estimators (one Monte Carlo draw eps[s] per sample, z_s = mu + sigma * eps_s):

* ``reparam_kl``  -- ``build_reparam_kl_loss_and_gradients`` (klqp.py:707-769):
  loss = -(mean_s sum_x scale*log p(x|z_s) - sum_z kl_scaling*KL(q||p)).
* ``reparam``     -- ``build_reparam_loss_and_gradients`` (klqp.py:642-704):
  loss = -(mean_s [log p(x|z_s) + log p(z_s)] - mean_s log q(z_s)).
* ``score``       -- ``build_score_loss_and_gradients`` (klqp.py:840-906):
  same loss; q-gradient = -mean_s grad log q(stop_grad z_s) * (p - q)_s.

Gradients are returned w.r.t. (mu, rho), i.e. through the softplus, which is
what ``tf.gradients(loss, var_list)`` yields for the two free variables.
"""
import numpy as np

from . import densities as dn

REPARAM_KL = 0
REPARAM = 1
SCORE = 2


def klqp_glm_loss_and_grads(model, mu, rho, eps, method=REPARAM_KL,
                            kl_scaling=1.0, latent_scale=1.0, dtype=np.float64):
    """Returns (loss, grad_mu, grad_rho, extras) for one ELBO-gradient eval.

    model: oracle.glm.GLM, mu/rho: [P], eps: [S, P].
    ``dtype`` sets the precision of the contraction (FP64 oracle or FP32 mirror).
    """
    mu = np.asarray(mu, np.float64)
    rho = np.asarray(rho, np.float64)
    eps = np.asarray(eps, np.float64)
    S = eps.shape[0]
    sigma = dn.softplus(rho)
    dsig_drho = dn.sigmoid(rho)
    Z = mu[None, :] + sigma[None, :] * eps
    if dtype == np.float32:
        Z = Z.astype(np.float32).astype(np.float64)
    ll = model.log_lik(Z, scaled=True, dtype=dtype)          # [S]
    lsc = np.broadcast_to(np.asarray(latent_scale, np.float64), mu.shape)
    extras = {"z": Z, "log_lik": ll}
    if method == REPARAM_KL:
        g = model.grad_log_lik(Z, scaled=True, dtype=dtype)  # [S, P]
        kls = np.broadcast_to(np.asarray(kl_scaling, np.float64), mu.shape)
        kl = dn.kl_normal_normal(mu, sigma, model.prior_loc, model.prior_scale)
        dkl_dmu, dkl_dsig = dn.kl_normal_normal_grads(mu, sigma, model.prior_loc, model.prior_scale)
        p_log_lik = ll.mean()
        kl_pen = float((kls * kl).sum())
        loss = -(p_log_lik - kl_pen)
        gmu = -g.mean(axis=0) + kls * dkl_dmu
        gsig = -(g * eps).mean(axis=0) + kls * dkl_dsig
        extras.update(p_log_lik=p_log_lik, kl_penalty=kl_pen)
    elif method == REPARAM:
        g = model.grad_log_lik(Z, scaled=True, dtype=dtype)
        lp_z = (lsc * dn.normal_log_prob(Z, model.prior_loc, model.prior_scale)).sum(axis=1)
        lq_z = (lsc * dn.normal_log_prob(Z, mu, sigma)).sum(axis=1)
        p_log_prob = (ll + lp_z).mean()
        q_log_prob = lq_z.mean()
        loss = -(p_log_prob - q_log_prob)
        # d/dz at fixed (mu, sigma)
        dfdz = g + lsc * dn.normal_grad_x(Z, model.prior_loc, model.prior_scale) \
            - lsc * dn.normal_grad_x(Z, mu, sigma)
        # direct dependence of -log q on (mu, sigma)
        dlq_dmu = (Z - mu) / sigma ** 2
        dlq_dsig = -1.0 / sigma + (Z - mu) ** 2 / sigma ** 3
        gmu = -(dfdz - lsc * dlq_dmu).mean(axis=0)
        gsig = -(dfdz * eps - lsc * dlq_dsig).mean(axis=0)
        extras.update(p_log_prob=p_log_prob, q_log_prob=q_log_prob)
    elif method == SCORE:
        lp_z = (lsc * dn.normal_log_prob(Z, model.prior_loc, model.prior_scale)).sum(axis=1)
        lq_z = (lsc * dn.normal_log_prob(Z, mu, sigma)).sum(axis=1)
        losses = ll + lp_z - lq_z                              # [S]
        loss = -losses.mean()
        dlq_dmu = lsc * (Z - mu) / sigma ** 2
        dlq_dsig = lsc * (-1.0 / sigma + (Z - mu) ** 2 / sigma ** 3)
        gmu = -(dlq_dmu * losses[:, None]).mean(axis=0)
        gsig = -(dlq_dsig * losses[:, None]).mean(axis=0)
        extras.update(losses=losses)
    else:
        raise ValueError(method)
    return float(loss), gmu, gsig * dsig_drho, extras


def default_learning_rate(global_step):
    """``tf.train.exponential_decay(0.1, global_step, 100, 0.9, staircase=True)``
    (``edward/inferences/variational_inference.py:83-93``), in FP32."""
    return np.float32(0.1) * np.float32(0.9) ** np.float32(global_step // 100)


class TFAdam:
    """``tf.train.AdamOptimizer`` apply rule (variational_inference.py:97,
    apply_gradients at 120-121): accumulators beta1_power/beta2_power start at
    beta1/beta2 and are multiplied after each apply;
    lr_t = lr * sqrt(1 - beta2_power) / (1 - beta1_power);
    m = b1 m + (1-b1) g;  v = b2 v + (1-b2) g^2;  p -= lr_t m / (sqrt(v) + eps)."""

    def __init__(self, n, beta1=0.9, beta2=0.999, epsilon=1e-8, dtype=np.float64):
        self.b1, self.b2, self.eps = beta1, beta2, epsilon
        self.m = np.zeros(n, dtype)
        self.v = np.zeros(n, dtype)
        self.b1p = np.float32(beta1)
        self.b2p = np.float32(beta2)
        self.dtype = dtype

    def apply(self, p, g, lr):
        dt = self.dtype
        g = np.asarray(g, dt)
        lr_t = dt(lr) * np.sqrt(dt(1) - dt(self.b2p)) / (dt(1) - dt(self.b1p))
        self.m = dt(self.b1) * self.m + dt(1 - self.b1) * g
        self.v = dt(self.b2) * self.v + dt(1 - self.b2) * g * g
        out = np.asarray(p, dt) - lr_t * self.m / (np.sqrt(self.v) + dt(self.eps))
        self.b1p = np.float32(self.b1p * np.float32(self.b1))
        self.b2p = np.float32(self.b2p * np.float32(self.b2))
        return out


def run_klqp_glm(model, mu0, rho0, n_iter, n_samples, seed, method=REPARAM_KL,
                 lr=None, eps_fn=None, dtype=np.float64):
    """Full optimisation loop in the shape of ``Inference.run``
    (``edward/inferences/inference.py:145-147``) with the default Adam.
    ``eps_fn(t) -> [S, P]`` supplies draws (defaults to the Philox stream)."""
    from .philox import normals, KIND_EPS
    mu = np.asarray(mu0, np.float64).copy()
    rho = np.asarray(rho0, np.float64).copy()
    P = mu.shape[0]
    opt = TFAdam(2 * P, dtype=np.float64)
    losses = []
    for t in range(n_iter):
        eps = eps_fn(t) if eps_fn else normals(seed, KIND_EPS, t, n_samples, P)
        loss, gmu, grho, _ = klqp_glm_loss_and_grads(model, mu, rho, eps, method, dtype=dtype)
        rate = default_learning_rate(t) if lr is None else lr
        theta = opt.apply(np.concatenate([mu, rho]), np.concatenate([gmu, grho]), rate)
        mu, rho = theta[:P], theta[P:]
        losses.append(loss)
    return mu, rho, np.array(losses)
