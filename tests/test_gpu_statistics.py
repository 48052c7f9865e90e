"""The reference's own statistical checks, run through the public API on the
GPU hot path (``ed.HMC`` on both engines, ``ed.KLqp``), plus tighter
many-chain versions of them against closed-form posteriors.

* Normal-Normal: x = 50 zeros, mu ~ N(0, 1), x ~ N(mu, 1); posterior
  N(0, 1/51) (``tests/inferences/klqp_test.py:14-44``,
  ``tests/inferences/hmc_test.py:14-46``), including the ``t`` / ``n_accept``
  checks and ``reset``.
* Bayesian linear regression, N = 40, D = 10, noise 0.1
  (``hmc_test.py:48-91``), against the conjugate posterior.

Monte Carlo tolerances: the many-chain checks use the final states of C
independent chains (i.i.d. draws from each chain's stationary law once the
burn-in is over), so the standard errors are exact: sd / sqrt(C) for a mean,
sd / sqrt(2C) for a standard deviation; the bar is 5 standard errors.
"""
import numpy as np
import pytest
import torch

from oracle.glm import conjugate_linreg_posterior

pytestmark = pytest.mark.gpu
POST_SD = np.sqrt(1.0 / 51.0)


def _normal_normal(ed):
    from edward_gb300.models import Normal
    x_data = np.zeros(50, np.float32)
    mu = Normal(loc=0.0, scale=1.0)
    x = Normal(loc=mu, scale=1.0, sample_shape=50)
    return mu, x, x_data


# ------------------------------------------------------------------ HMC

@pytest.mark.parametrize("engine", ["tc", "simt"])
@pytest.mark.parametrize("default", [False, True])
def test_hmc_normal_normal_reference_check(cuda, engine, default):
    """hmc_test.py:14-46 as written: one chain, default step size 0.25 and
    2 leapfrog steps, 2,000 (given store) or 10,000 (default store) samples."""
    import edward_gb300 as ed
    from edward_gb300.models import Empirical
    ed.set_seed(42)
    mu, x, x_data = _normal_normal(ed)
    n_samples = 2000
    if not default:
        qmu = Empirical(params=ed.Variable(np.ones(n_samples, np.float32)))
        inference = ed.HMC({mu: qmu}, data={x: x_data})
    else:
        inference = ed.HMC([mu], data={x: x_data})
        qmu = inference.latent_vars[mu]
    inference.run(engine=engine)
    inference.check_errors()
    assert inference.engine == engine
    np.testing.assert_allclose(float(qmu.mean()), 0.0, rtol=1e-1, atol=1e-1)
    np.testing.assert_allclose(float(qmu.stddev()), POST_SD, rtol=1e-1, atol=1e-1)
    assert inference.t == (n_samples if not default else 10000)
    assert inference.n_accept > 0.1
    inference.reset()
    assert inference.t == 0
    assert inference.n_accept == 0


@pytest.mark.parametrize("engine", ["tc", "simt"])
def test_hmc_normal_normal_many_chains(cuda, engine):
    """4,096 chains from mu = 1 for 600 iterations: the final states match
    N(0, 1/51) in mean and standard deviation within 5 standard errors."""
    import edward_gb300 as ed
    from edward_gb300.models import Empirical
    ed.set_seed(7)
    mu, x, x_data = _normal_normal(ed)
    C, T = 4096, 600
    qmu = Empirical(params=ed.Variable(np.ones((T, C), np.float32)), n_chains=C)
    inference = ed.HMC({mu: qmu}, data={x: x_data}, n_chains=C)
    inference.run(engine=engine, n_print=0)
    inference.check_errors()
    final = qmu.params[-1].double().cpu().numpy()
    n = final.size
    assert abs(final.mean()) < 5 * POST_SD / np.sqrt(n)
    assert abs(final.std() - POST_SD) < 5 * POST_SD / np.sqrt(2 * n)
    acc = inference.n_accept.double().mean().item() / T
    assert acc > 0.1


def _linreg_data(seed=0, N=40, D=10, noise=0.1):
    rng = np.random.default_rng(seed)
    w_true = rng.standard_normal(D)
    X = rng.standard_normal((N, D))
    y = X @ w_true + rng.normal(0, noise, size=N)
    return X.astype(np.float32), y.astype(np.float32), w_true


@pytest.mark.parametrize("engine", ["tc", "simt"])
def test_hmc_linear_regression_reference_check(cuda, engine):
    """hmc_test.py:48-91 as written: placeholder X, step size 0.01, 2,000
    samples of (w, b); the posterior means are near w_true and 0."""
    import edward_gb300 as ed
    from edward_gb300.models import Empirical, Normal
    ed.set_seed(1)
    N, D = 40, 10
    X_train, y_train, w_true = _linreg_data()
    X = ed.placeholder(np.float32, [N, D])
    w = Normal(loc=ed.zeros(D), scale=ed.ones(D))
    b = Normal(loc=ed.zeros(1), scale=ed.ones(1))
    y = Normal(loc=ed.dot(X, w) + b, scale=0.1 * np.ones(N, np.float32))
    n_samples = 2000
    qw = Empirical(ed.Variable(np.zeros([n_samples, D], np.float32)))
    qb = Empirical(ed.Variable(np.zeros([n_samples, 1], np.float32)))
    inference = ed.HMC({w: qw, b: qb}, data={X: X_train, y: y_train})
    inference.run(step_size=0.01, engine=engine)
    inference.check_errors()
    np.testing.assert_allclose(qw.mean().cpu().numpy(), w_true, rtol=5e-1, atol=5e-1)
    np.testing.assert_allclose(qb.mean().cpu().numpy(), [0.0], rtol=5e-1, atol=5e-1)
    assert inference.t == n_samples
    assert inference.n_accept > 0.1
    inference.reset()
    assert inference.t == 0 and inference.n_accept == 0


@pytest.mark.parametrize("engine", ["tc", "simt"])
def test_hmc_linear_regression_conjugate_posterior(cuda, engine):
    """The same model with 4,096 chains started at exact draws from the
    closed-form conjugate posterior N(m, S): a correct HMC kernel leaves that
    law invariant, so after 100 iterations of 5 leapfrog steps of 0.01 the
    chains' states, whitened (z -> L^-1 (z - m), S = L L^T), still have mean 0
    and covariance I within 5 standard errors (1/sqrt(C) for the mean,
    sqrt((1 + [i = j]) / C) for covariance entries).  The chains must also have
    moved: the whitened displacement from the start has RMS above 1 (an
    identity map would leave the law invariant too), and the acceptance rate
    is above one half."""
    import edward_gb300 as ed
    from edward_gb300.models import Empirical, Normal
    ed.set_seed(3)
    N, D, C, T = 40, 10, 4096, 100
    X_train, y_train, _ = _linreg_data()
    mean, cov = conjugate_linreg_posterior(X_train, y_train, 0.1)
    Lc = np.linalg.cholesky(cov)
    w = Normal(loc=ed.zeros(D), scale=ed.ones(D))
    b = Normal(loc=ed.zeros(1), scale=ed.ones(1))
    y = Normal(loc=ed.dot(X_train, w) + b, scale=0.1 * np.ones(N, np.float32))
    z0 = mean + (Lc @ np.random.default_rng(5).standard_normal((D + 1, C))).T
    w0 = np.zeros((T, C, D), np.float32)
    b0 = np.zeros((T, C, 1), np.float32)
    w0[0] = z0[:, :D]
    b0[0] = z0[:, D:]
    qw = Empirical(ed.Variable(w0), n_chains=C)
    qb = Empirical(ed.Variable(b0), n_chains=C)
    inference = ed.HMC({w: qw, b: qb}, data={y: y_train}, n_chains=C)
    inference.run(step_size=0.01, n_steps=5, engine=engine, n_print=0)
    inference.check_errors()
    Zf = np.concatenate([qw.params[-1].double().cpu().numpy(),
                         qb.params[-1].double().cpu().numpy()], axis=1)
    W = np.linalg.solve(Lc, (Zf - mean).T).T
    W0 = np.linalg.solve(Lc, (z0.astype(np.float32).astype(np.float64) - mean).T).T
    P = D + 1
    assert np.all(np.abs(W.mean(axis=0)) < 5 / np.sqrt(C)), W.mean(axis=0)
    emp = np.cov(W.T, bias=True)
    se = np.sqrt((1 + np.eye(P)) / C)
    assert np.all(np.abs(emp - np.eye(P)) < 5 * se), np.abs(emp - np.eye(P)).max()
    assert np.sqrt(((W - W0) ** 2).mean()) > 1.0
    assert inference.n_accept.double().mean().item() / T > 0.5


# ------------------------------------------------------------------ KLqp

@pytest.mark.parametrize("default", [False, True])
def test_klqp_normal_normal_reference_check(cuda, default):
    """klqp_test.py:14-44 as written: 5,000 iterations of ed.KLqp (analytic KL,
    default Adam and learning-rate schedule); q's mean and standard deviation
    match N(0, 1/51); t == n_iter; reset zeroes t and re-initialises the
    optimizer state."""
    import edward_gb300 as ed
    from edward_gb300.models import Normal
    ed.set_seed(42)
    mu, x, x_data = _normal_normal(ed)
    if not default:
        qmu_loc = ed.Variable(np.float32(np.random.default_rng(0).standard_normal()))
        qmu_scale = ed.softplus(ed.Variable(np.float32(np.random.default_rng(1).standard_normal())))
        qmu = Normal(loc=qmu_loc, scale=qmu_scale)
        inference = ed.KLqp({mu: qmu}, data={x: x_data})
    else:
        inference = ed.KLqp([mu], data={x: x_data})
        qmu = inference.latent_vars[mu]
    inference.run(n_iter=5000, n_print=0)
    m, s = float(qmu.mean()), float(qmu.stddev())
    np.testing.assert_allclose(m, 0.0, rtol=0.1, atol=0.6)
    np.testing.assert_allclose(s, POST_SD, rtol=0.15, atol=0.5)
    # the tighter bars the FP64 oracle meets on this problem
    assert abs(m) < 0.05
    assert abs(s - POST_SD) < 0.02
    assert inference.t == inference.n_iter
    old = inference._slots.detach().clone()
    inference.reset()
    assert inference.t == 0
    assert not torch.equal(old, inference._slots)
