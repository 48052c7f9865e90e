"""Model parameters (the reference's p_vars: trainable variables of the model
that are not latent, ``klqp.py:902-904``): KLqp fits them with the pathwise
gradient of the loss while it fits q for the latents.

* ``klqp_test.py:46-56``: x = [0,1,0,0,0,0,0,0,0,1] ~ Bernoulli(probs =
  sigmoid(Variable(0.5))), no latent variables, 50 iterations of the default
  Adam: sigmoid(Variable) reaches the maximum-likelihood 0.2.
* A logistic regression with latent w and a model-parameter intercept b: the
  fused step's loss and gradients against the FP64 oracle with the same draws.
"""
import numpy as np
import pytest
import torch

from oracle import densities as dn
from oracle.glm import GLM, synthetic_logreg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cls_name", ["KLqp", "ReparameterizationKLqp", "ReparameterizationKLKLqp",
                                      "ScoreKLqp"])
def test_model_parameter_reference_check(cuda, cls_name):
    import edward_gb300 as ed
    from edward_gb300.models import Bernoulli
    x_data = np.array([0, 1, 0, 0, 0, 0, 0, 0, 0, 1])
    v = ed.Variable(0.5)
    p = ed.sigmoid(v)
    x = Bernoulli(probs=p, sample_shape=10)
    inference = getattr(ed, cls_name)({}, data={x: x_data})
    inference.run(n_iter=50, n_print=0)
    np.testing.assert_allclose(float(torch.sigmoid(v.value)), 0.2, rtol=5e-2, atol=5e-2)
    assert inference.t == 50


def test_latent_and_model_parameter_gradients(cuda):
    """w ~ N(0, 1) latent with q = N(mu, softplus(rho)), b a model parameter:
    loss = -(mean_s log p(y | X z_s + b) - KL(q || p)), d loss / d b =
    -mean_s d log p / d b at the same draws, d loss / d (mu, rho) as for any
    latent; all within 1e-5 of the FP64 oracle."""
    import edward_gb300 as ed
    from edward_gb300.models import Bernoulli, Normal
    N, D, S = 3000, 6, 5
    X, y, _, _ = synthetic_logreg(N, D, seed=12)
    w = Normal(loc=ed.zeros(D), scale=ed.ones(D))
    b = ed.Variable(np.float32(0.3))
    yv = Bernoulli(logits=ed.dot(X, w) + b)
    inf = ed.KLqp([w], data={yv: y})
    inf.initialize(n_samples=S, n_iter=10, n_print=0)
    P = D + 1
    rng = np.random.default_rng(3)
    mu = (rng.standard_normal(D) * 0.3).astype(np.float32)
    rho = (rng.standard_normal(D) * 0.3 - 1).astype(np.float32)
    inf._mu[:D].copy_(torch.as_tensor(mu))
    inf._rho[:D].copy_(torch.as_tensor(rho))
    eps = rng.standard_normal((S, P)).astype(np.float32)
    loss, gmu, grho = inf.loss_and_gradients(eps)
    m = GLM(X.astype(np.float32), y.astype(np.float32), bias=True)
    sig = dn.softplus(rho.astype(np.float64))
    Z = np.concatenate([mu[None] + sig[None] * eps[:, :D], np.full((S, 1), 0.3)], axis=1)
    ll = m.log_lik(Z)
    g = m.grad_log_lik(Z)
    kl = dn.kl_normal_normal(mu.astype(np.float64), sig, 0.0, 1.0).sum()
    e_loss = -(ll.mean() - kl)
    dkl_mu, dkl_sig = dn.kl_normal_normal_grads(mu.astype(np.float64), sig, 0.0, 1.0)
    e_gmu = np.concatenate([-g[:, :D].mean(0) + dkl_mu, [-g[:, D].mean()]])
    e_grho = (-(g[:, :D] * eps[:, :D]).mean(0) + dkl_sig) * dn.sigmoid(rho.astype(np.float64))
    gmu, grho = gmu.cpu().numpy(), grho.cpu().numpy()
    assert abs(loss - e_loss) <= 1e-5 * abs(e_loss)
    np.testing.assert_allclose(gmu, e_gmu, rtol=1e-5, atol=1e-5 * np.abs(e_gmu).max())
    np.testing.assert_allclose(grho[:D], e_grho, rtol=1e-5, atol=1e-5 * np.abs(e_grho).max())
    assert grho[D] == 0.0
    # an update moves b by the Adam step of its gradient and leaves its rho alone
    inf._step(apply=True, eps=torch.as_tensor(eps, device=cuda))
    assert float(inf._rho[D]) == 0.0
    assert abs(float(b.value) - 0.3) > 1e-4


@pytest.mark.parametrize("cls_name", ["ReparameterizationKLqp", "ReparameterizationKLKLqp",
                                      "ScoreKLqp"])
def test_model_parameter_gradient_every_method(cuda, cls_name):
    """Whatever estimator fits q, the model parameter's gradient is the pathwise
    -mean_s d log p(y | X z_s + b) / d b at the step's draws (``klqp.py:902-904``
    differentiates the loss itself); within 1e-5 of the FP64 oracle."""
    import edward_gb300 as ed
    from edward_gb300.models import Bernoulli, Normal
    N, D, S = 2000, 5, 4
    X, y, _, _ = synthetic_logreg(N, D, seed=21)
    w = Normal(loc=ed.zeros(D), scale=ed.ones(D))
    b = ed.Variable(np.float32(-0.2))
    yv = Bernoulli(logits=ed.dot(X, w) + b)
    inf = getattr(ed, cls_name)([w], data={yv: y})
    inf.initialize(n_samples=S, n_iter=10, n_print=0)
    P = D + 1
    rng = np.random.default_rng(5)
    eps = rng.standard_normal((S, P)).astype(np.float32)
    mu = inf._mu[:D].cpu().numpy().astype(np.float64)
    rho = inf._rho[:D].cpu().numpy().astype(np.float64)
    _, gmu, grho = inf.loss_and_gradients(eps)
    m = GLM(X.astype(np.float32), y.astype(np.float32), bias=True)
    Z = np.concatenate([mu[None] + dn.softplus(rho)[None] * eps[:, :D], np.full((S, 1), -0.2)],
                       axis=1)
    e_gb = -m.grad_log_lik(Z)[:, D].mean()
    got = float(gmu[D])
    assert abs(got - e_gb) <= 1e-5 * max(1.0, abs(e_gb)), (got, e_gb)
    assert float(grho[D]) == 0.0
