"""Constrained latents under auto_transform (Beta-Bernoulli, Gamma-Poisson,
Dirichlet-Categorical): HMC and KLqp in the unconstrained space against the FP64
oracle with the same draws, and the reference's Beta-Bernoulli posterior checks
(tests/inferences/inference_auto_transform_test.py:163-217)."""
import numpy as np
import pytest
import torch

from oracle import expfam as ef
from oracle import hmc as ohmc

pytestmark = pytest.mark.gpu

X_OBS = np.asarray([0, 0, 1, 1, 0, 0, 0, 0, 0, 1], dtype=np.int32)


def _model(ed, family, rng):
    from edward_gb300.models import Bernoulli, Beta, Categorical, Dirichlet, Gamma, Poisson
    if family == ef.BETA:
        z = Beta(1.5, 2.0)
        x = Bernoulli(probs=z, sample_shape=10)
        return z, x, X_OBS, (1.5, 2.0), 1
    if family == ef.GAMMA:
        z = Gamma(2.0, 0.5)
        x = Poisson(rate=z, sample_shape=12)
        data = rng.poisson(3.0, 12).astype(np.float32)
        return z, x, data, (2.0, 0.5), 1
    alpha = np.array([1.0, 2.0, 0.5, 3.0], np.float32)
    z = Dirichlet(alpha)
    x = Categorical(probs=z, sample_shape=30)
    data = rng.integers(0, 4, 30)
    return z, x, data, alpha, 3


@pytest.mark.parametrize("family", [ef.BETA, ef.GAMMA, ef.DIRICHLET])
def test_expfam_hmc_matches_oracle(cuda, family):
    """FP32 chain state, momenta and gradients, FP64 log-joint sums and
    energy difference; the oracle runs the same leapfrog in FP32 on its FP64
    log joint and gradient, so the samples agree to FP32 rounding (1e-5)."""
    import edward_gb300 as ed
    from edward_gb300.models import Empirical
    rng = np.random.default_rng(family)
    z, x, data, prior, K = _model(ed, family, rng)
    stats = ef.sufficient_stats(family, data, K + 1)
    C, n, L, eps = 6, 3, 4, 0.2
    shape = (20, C, K) if family == ef.DIRICHLET else (20, C)
    u0 = rng.standard_normal((C, K)) * 0.5
    init = np.zeros(shape, np.float32)
    init[0] = u0.reshape(shape[1:]).astype(np.float32)
    qz = Empirical(ed.Variable(init), n_chains=C)
    inf = ed.HMC({z: qz}, data={x: data}, n_chains=C)
    inf.initialize(step_size=eps, n_steps=L, n_print=0)
    r = rng.standard_normal((n, C, K)).astype(np.float32)
    u = rng.random((n, C))
    inf.run_iterations(n, r_override=torch.as_tensor(r, device=cuda),
                       u_override=torch.as_tensor(u, device=cuda))

    def lj_grad(U):
        return ef.log_joint(family, prior, stats, U), ef.grad_log_joint(family, prior, stats, U)

    zc = u0.astype(np.float32)
    lj0, g0 = lj_grad(zc)
    worst = 0.0
    for t in range(n):
        # the step size reaches the kernel as the FP32 edg_hmc_t::step_size
        out = ohmc.hmc_step(lj_grad, zc, g0, lj0, r[t], u[t], float(np.float32(eps)), L,
                            dtype=np.float32)
        zc, g0, lj0 = out["z"], out["g"], out["lj"]
        got = inf._samples[t].cpu().numpy()
        assert got.dtype == np.float32
        np.testing.assert_allclose(got, zc, rtol=1e-5, atol=1e-6)
        worst = max(worst, float(np.abs(got - zc).max()))
    print(f"expfam family {family}: max |u_gpu - u_oracle| = {worst:.2e}")
    assert inf.t == n


@pytest.mark.parametrize("family", [ef.BETA, ef.GAMMA, ef.DIRICHLET])
def test_expfam_klqp_step_matches_oracle(cuda, family):
    import edward_gb300 as ed
    from edward_gb300.models import Normal
    rng = np.random.default_rng(10 + family)
    z, x, data, prior, K = _model(ed, family, rng)
    stats = ef.sufficient_stats(family, data, K + 1)
    shape = (K,) if family == ef.DIRICHLET else ()
    mu0 = (rng.standard_normal(shape) * 0.3).astype(np.float32)
    rho0 = (rng.standard_normal(shape) * 0.3 - 1.0).astype(np.float32)
    qz = Normal(loc=ed.Variable(mu0), scale=ed.softplus(ed.Variable(rho0)))
    inf = ed.KLqp({z: qz}, data={x: data})
    S = 7
    inf.initialize(n_samples=S, auto_transform=True)
    eps = rng.standard_normal((S, K)).astype(np.float32)
    loss, gmu, grho = inf.loss_and_gradients(eps)
    l0, m0, r0 = ef.klqp_loss_and_grads(family, prior, stats, mu0.reshape(-1), rho0.reshape(-1),
                                        eps)
    assert abs(loss - l0) <= 1e-5 * max(1.0, abs(l0))
    np.testing.assert_allclose(gmu.cpu().numpy(), m0, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(grho.cpu().numpy(), r0, rtol=1e-5, atol=1e-6)


def test_hmc_beta_bernoulli_posterior(cuda):
    """tests/inferences/inference_auto_transform_test.py:163-188."""
    import edward_gb300 as ed
    from edward_gb300.models import Bernoulli, Beta, Empirical
    ed.set_seed(124125)
    z = Beta(1., 1.)
    xs = Bernoulli(probs=z, sample_shape=10)
    qz = Empirical(ed.Variable(np.random.default_rng(0).random(1000).astype(np.float32)))
    inference = ed.HMC({z: qz}, data={xs: X_OBS})
    inference.run(step_size=1.0, n_steps=5, auto_transform=True, n_print=0)
    s = qz.params.double()
    a, b = 1. + X_OBS.sum(), 1. + (1 - X_OBS).sum()
    assert abs(float(s.mean()) - a / (a + b)) < 5e-2
    assert abs(float(s.var(unbiased=False)) - a * b / ((a + b) ** 2 * (a + b + 1))) < 1e-2


def test_klqp_beta_bernoulli_posterior(cuda):
    """tests/inferences/inference_auto_transform_test.py:190-217."""
    import edward_gb300 as ed
    from edward_gb300.models import Bernoulli, Beta, Normal
    ed.set_seed(124125)
    z = Beta(1., 1.)
    xs = Bernoulli(probs=z, sample_shape=10)
    qz = Normal(loc=ed.Variable(np.float32(np.random.randn())),
                scale=ed.softplus(ed.Variable(np.float32(np.random.randn()))))
    inference = ed.KLqp({z: qz}, data={xs: X_OBS})
    inference.run(n_iter=500, auto_transform=True, n_print=0)
    u = qz.loc.value.double() + torch.nn.functional.softplus(qz.scale.args[0].value.double()) * \
        torch.randn(100000, dtype=torch.float64, device=cuda)
    zs = inference.transformations[z](u)
    a, b = 1. + X_OBS.sum(), 1. + (1 - X_OBS).sum()
    assert abs(float(zs.mean()) - a / (a + b)) < 5e-2
    assert abs(float(zs.var()) - a * b / ((a + b) ** 2 * (a + b + 1))) < 1e-2


@pytest.mark.parametrize("family", [ef.GAMMA, ef.DIRICHLET])
def test_hmc_conjugate_posteriors(cuda, family):
    """Many chains: posterior mean of z against the conjugate posterior."""
    import edward_gb300 as ed
    from edward_gb300.models import Empirical
    ed.set_seed(3)
    rng = np.random.default_rng(3)
    z, x, data, prior, K = _model(ed, family, rng)
    C, T = 64, 400
    shape = (T, C, K) if family == ef.DIRICHLET else (T, C)
    qz = Empirical(ed.Variable(np.zeros(shape, np.float32)), n_chains=C)
    inference = ed.HMC({z: qz}, data={x: data}, n_chains=C)
    inference.run(step_size=0.2, n_steps=5, n_print=0)
    zs = qz.params[100:].double().reshape(-1, K + 1 if family == ef.DIRICHLET else 1)
    if family == ef.GAMMA:
        a, r = prior[0] + data.sum(), prior[1] + data.size
        assert abs(float(zs.mean()) - a / r) < 0.05 * a / r
    else:
        post = prior + np.bincount(data, minlength=4)
        np.testing.assert_allclose(zs.mean(0).cpu().numpy(), post / post.sum(), atol=0.02)


@pytest.mark.parametrize("family", [ef.BETA, ef.GAMMA])
def test_expfam_klqp_on_support_matches_oracle(cuda, family):
    """auto_transform=False: q fitted on the latent's support itself (z = u, no
    Jacobian); with every draw inside the support, loss and gradients agree
    with the FP64 oracle to 1e-5."""
    import edward_gb300 as ed
    from edward_gb300.models import Normal
    rng = np.random.default_rng(20 + family)
    z, x, data, prior, K = _model(ed, family, rng)
    stats = ef.sufficient_stats(family, data, K + 1)
    mu0 = np.float32(0.4 if family == ef.BETA else 3.0)
    rho0 = np.float32(-3.0 if family == ef.BETA else -1.0)
    qz = Normal(loc=ed.Variable(mu0), scale=ed.softplus(ed.Variable(rho0)))
    inf = ed.KLqp({z: qz}, data={x: data})
    S = 6
    inf.initialize(n_samples=S, auto_transform=False)
    eps = np.clip(rng.standard_normal((S, 1)), -2.0, 2.0).astype(np.float32)
    loss, gmu, grho = inf.loss_and_gradients(eps)
    l0, m0, r0 = ef.klqp_loss_and_grads(family, prior, stats, [mu0], [rho0], eps,
                                        transform=False)
    assert np.isfinite(l0)
    assert abs(loss - l0) <= 1e-5 * max(1.0, abs(l0))
    np.testing.assert_allclose(gmu.cpu().numpy(), m0, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(grho.cpu().numpy(), r0, rtol=1e-5, atol=1e-6)


def test_klqp_auto_transform_false_gives_nan(cuda):
    """tests/inferences/inference_auto_transform_test.py:46-63: a latent with a
    nonnegative support fitted by a Normal q without auto_transform; q's draws
    leave the support and the loss becomes NaN (numerical failure is not an
    error).  With auto_transform the same fit stays finite."""
    import edward_gb300 as ed
    from edward_gb300.models import Gamma, Normal
    for auto, expect_nan in ((False, True), (True, False)):
        ed.set_seed(42)
        x = Gamma(2.0, 4.0)
        rng = np.random.default_rng(0)
        qx = Normal(loc=ed.Variable(np.float32(rng.standard_normal())),
                    scale=ed.softplus(ed.Variable(np.float32(rng.standard_normal()))))
        inference = ed.KLqp({x: qx})
        inference.initialize(auto_transform=auto, n_samples=5, n_iter=150)
        for _ in range(inference.n_iter):
            info_dict = inference.update()
        assert bool(np.isnan(info_dict["loss"])) == expect_nan, (auto, info_dict)


def test_expfam_dirichlet_largest_supported_size(cuda):
    """A Dirichlet over 33 categories (the largest unconstrained dimension, 32):
    one KLqp step's loss and gradients and one HMC iteration against the
    oracle with the same draws."""
    import edward_gb300 as ed
    from edward_gb300.models import Categorical, Dirichlet, Empirical, Normal
    rng = np.random.default_rng(33)
    Kc = 33
    alpha = rng.uniform(0.5, 3.0, Kc).astype(np.float32)
    data = rng.integers(0, Kc, 200)
    stats = ef.sufficient_stats(ef.DIRICHLET, data, Kc)
    K = Kc - 1
    # KLqp
    z = Dirichlet(alpha)
    x = Categorical(probs=z, sample_shape=200)
    mu0 = (rng.standard_normal(K) * 0.3).astype(np.float32)
    rho0 = (rng.standard_normal(K) * 0.3 - 1.0).astype(np.float32)
    qz = Normal(loc=ed.Variable(mu0), scale=ed.softplus(ed.Variable(rho0)))
    inf = ed.KLqp({z: qz}, data={x: data})
    S = 9
    inf.initialize(n_samples=S, auto_transform=True)
    eps = rng.standard_normal((S, K)).astype(np.float32)
    loss, gmu, grho = inf.loss_and_gradients(eps)
    l0, m0, r0 = ef.klqp_loss_and_grads(ef.DIRICHLET, alpha, stats, mu0, rho0, eps)
    assert abs(loss - l0) <= 1e-5 * max(1.0, abs(l0))
    np.testing.assert_allclose(gmu.cpu().numpy(), m0, rtol=1e-5, atol=1e-5 * np.abs(m0).max())
    np.testing.assert_allclose(grho.cpu().numpy(), r0, rtol=1e-5, atol=1e-5 * np.abs(r0).max())
    # HMC
    z2 = Dirichlet(alpha)
    x2 = Categorical(probs=z2, sample_shape=200)
    C, L, step = 5, 3, 0.05
    u0 = (rng.standard_normal((C, K)) * 0.3).astype(np.float32)
    init = np.zeros((4, C, K), np.float32)
    init[0] = u0
    qz2 = Empirical(ed.Variable(init), n_chains=C)
    hmc = ed.HMC({z2: qz2}, data={x2: data}, n_chains=C)
    hmc.initialize(step_size=step, n_steps=L, n_print=0)
    r = rng.standard_normal((1, C, K)).astype(np.float32)
    u = rng.random((1, C))
    hmc.run_iterations(1, r_override=torch.as_tensor(r, device=cuda),
                       u_override=torch.as_tensor(u, device=cuda))

    def lj_grad(U):
        return (ef.log_joint(ef.DIRICHLET, alpha, stats, U),
                ef.grad_log_joint(ef.DIRICHLET, alpha, stats, U))
    lj0, g0 = lj_grad(u0)
    out = ohmc.hmc_step(lj_grad, u0, g0, lj0, r[0], u[0], float(np.float32(step)), L,
                        dtype=np.float32)
    got = hmc._samples[0].cpu().numpy()
    np.testing.assert_allclose(got, out["z"], rtol=1e-5, atol=1e-5 * np.abs(out["z"]).max())
